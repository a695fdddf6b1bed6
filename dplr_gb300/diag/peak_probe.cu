// peak_probe.cu -- arithmetic and copy peaks of the GPU the library runs on.
//
// FP64 FMA (DFMA), FP64 tensor MMA (mma.sync m8n8k4 f64), FP32 FMA and a
// streaming double4 copy.  The FP64 numbers are the roofline denominators
// of the FP64 kernels (MEASURED_PEAKS.json holds only the copy bandwidth
// and the bf16 GEMM rate).  Run with:  python -m dplr_gb300.diag.peak_probe
#include <cstdio>
#include <cuda_runtime.h>
#define CK(x) do{cudaError_t e=(x); if(e!=cudaSuccess){printf("ERR %s line %d: %s\n",#x,__LINE__,cudaGetErrorString(e)); return 1;}}while(0)

__global__ void k_dfma(double* out, int iters, double a, double b){
  double c0=threadIdx.x,c1=c0+1,c2=c0+2,c3=c0+3,c4=c0+4,c5=c0+5,c6=c0+6,c7=c0+7;
  for(int i=0;i<iters;i++){
    c0=fma(c0,a,b);c1=fma(c1,a,b);c2=fma(c2,a,b);c3=fma(c3,a,b);
    c4=fma(c4,a,b);c5=fma(c5,a,b);c6=fma(c6,a,b);c7=fma(c7,a,b);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=c0+c1+c2+c3+c4+c5+c6+c7;
}
__global__ void k_ffma(float* out, int iters, float a, float b){
  float c0=threadIdx.x,c1=c0+1,c2=c0+2,c3=c0+3,c4=c0+4,c5=c0+5,c6=c0+6,c7=c0+7;
  for(int i=0;i<iters;i++){
    c0=fmaf(c0,a,b);c1=fmaf(c1,a,b);c2=fmaf(c2,a,b);c3=fmaf(c3,a,b);
    c4=fmaf(c4,a,b);c5=fmaf(c5,a,b);c6=fmaf(c6,a,b);c7=fmaf(c7,a,b);
  }
  out[blockIdx.x*blockDim.x+threadIdx.x]=c0+c1+c2+c3+c4+c5+c6+c7;
}
__global__ void k_dmma(double* out, int iters){
  double a = 1.0 + threadIdx.x*1e-3, b = 0.5;
  double d[4][2];
  for(int j=0;j<4;j++){d[j][0]=0;d[j][1]=0;}
  for(int i=0;i<iters;i++){
    #pragma unroll
    for(int j=0;j<4;j++){
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
        : "+d"(d[j][0]), "+d"(d[j][1]) : "d"(a), "d"(b));
    }
  }
  double s=0; for(int j=0;j<4;j++) s+=d[j][0]+d[j][1];
  out[blockIdx.x*blockDim.x+threadIdx.x]=s;
}
__global__ void k_copy(const double4_32a* __restrict__ src, double4_32a* __restrict__ dst, size_t n){
  size_t i = blockIdx.x*(size_t)blockDim.x+threadIdx.x, st=(size_t)gridDim.x*blockDim.x;
  for(; i<n; i+=st) dst[i]=src[i];
}
int main(){
  int dev=0; cudaDeviceProp p; CK(cudaGetDeviceProperties(&p,dev));
  printf("name %s sms %d cc %d.%d l2 %d smem/blk optin %zu\n", p.name,p.multiProcessorCount,p.major,p.minor,p.l2CacheSize,p.sharedMemPerBlockOptin);
  int sms=p.multiProcessorCount;
  double* dout; CK(cudaMalloc(&dout, sizeof(double)*sms*8*1024));
  cudaEvent_t e0,e1; cudaEventCreate(&e0); cudaEventCreate(&e1); float ms;
  for(int blocksPerSm : {4, 8}){
    int iters=4096; int nb=sms*blocksPerSm, nt=256;
    k_dfma<<<nb,nt>>>(dout,16,1.0000001,1e-9); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_dfma<<<nb,nt>>>(dout,iters,1.0000001,1e-9); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms,e0,e1);
    double fl=2.0*8*iters*(double)nb*nt; printf("DFMA bps=%d: %.3f ms  %.3f TFLOP/s\n",blocksPerSm,ms,fl/ms/1e9);
    k_ffma<<<nb,nt>>>((float*)dout,16,1.0000001f,1e-9f); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_ffma<<<nb,nt>>>((float*)dout,iters*16,1.0000001f,1e-9f); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms,e0,e1);
    fl=2.0*8*iters*16*(double)nb*nt; printf("FFMA bps=%d: %.3f ms  %.3f TFLOP/s\n",blocksPerSm,ms,fl/ms/1e9);
    k_dmma<<<nb,nt>>>(dout,16); CK(cudaDeviceSynchronize());
    cudaEventRecord(e0); k_dmma<<<nb,nt>>>(dout,iters/4); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms,e0,e1);
    fl=2.0*8*8*4*4*(double)(iters/4)*nb*(nt/32); printf("DMMA bps=%d: %.3f ms  %.3f TFLOP/s\n",blocksPerSm,ms,fl/ms/1e9);
  }
  size_t n = (size_t)1<<27; // 128M double4_32a? no: 2^27 double4_32a = 4 GiB; use 2^26 = 2 GiB each
  n = (size_t)1<<26;
  double4_32a *a,*b; CK(cudaMalloc(&a,n*sizeof(double4_32a))); CK(cudaMalloc(&b,n*sizeof(double4_32a)));
  CK(cudaMemset(a,0,n*sizeof(double4_32a)));
  for(int r=0;r<3;r++){
    cudaEventRecord(e0); k_copy<<<sms*8,256>>>(a,b,n); cudaEventRecord(e1); CK(cudaEventSynchronize(e1));
    cudaEventElapsedTime(&ms,e0,e1); printf("copy %.3f ms %.1f GB/s\n",ms, 2.0*n*sizeof(double4_32a)/ms/1e6);
  }
  printf("done\n");
  return 0;
}
