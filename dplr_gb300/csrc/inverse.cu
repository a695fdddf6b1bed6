// inverse.cu -- dplrgeinv on the GPU: B := inv(A) as a PLR tree in DPLR's
// own representation (DPLR src/dplrinv.c:93-450 with src/dplrprk.c:21).
//
// DPLR builds B post-order: at node q it forms, from the children's
// inverses, u1 = A1^-1 U1, u2 = A2^-1 U2, v1 = A2^-T V1, v2 = A1^-T V2 and
// Y = [[S1^-1, V1^T u2], [V2^T u1, S2^-1]]^-1; then
//   B.ne = (-u1 Y11, v1),  B.sw = (-u2 Y22, v2)        (normalised pairs)
//   nw += (-u1 Y12) v2^T,  se += (-u2 Y21) v1^T        (dplrgeprk)
// where dplrgeprk appends the normalised correction columns, restricted to
// each block, to every low-rank block below q and adds them to the leaves;
// nothing is ever recompressed.
//
// The GPU computes the same objects from the Woodbury factorisation
// (factor.cu): u = Z, v = Zt, and Y = X^-1 = K^-1 S because X = S^-1 K.
// Per level l, one launch forms  P_l = -Z_l K^-1 S  for all nodes (rows of
// the nw child hold [-u1 Y11 | -u1 Y12], rows of the se child hold
// [-u2 Y21 | -u2 Y22]); one launch normalises every correction generator;
// one launch normalises every column of every block of B (own columns and
// all appended ancestor groups, each with the node's own threshold, which
// is what dplrgeprk's eps/2, eps/4 recursion amounts to); one launch
// assembles the leaves.  The host then replays DPLR's structural steps on
// B (type checks, dplrinilr, dplrresizelr growth) and copies the values
// in, so rank, capacity and column order match DPLR exactly.
#include "factor.cuh"

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

namespace dg {

struct ColJob {
    long long us, vs;      // source column starts
    long long ud, vd;      // destination column starts
    long long sd;          // destination of the singular value
    long long mult;        // index of the multiplier (d of a generator), -1 for 1
    double eps2;
    double usign;          // sign folded into u when the pair is kept
    int len;
};

struct AncTerm {
    long long goff;        // offset of Gu_la / Gv_la (same in both pools)
    long long doff;        // first d of the generator
    int k;
};

struct LeafJob {
    long long src, dst;    // leaf inverse offset, staging offset
    int row0, b, first, count;
};

// One CTA per column pair: norms, singular value, scaled (or raw) copies.
__global__ void colpair_kernel(const ColJob *__restrict__ jobs, const double *__restrict__ usrc,
                               const double *__restrict__ vsrc, const double *__restrict__ mult,
                               double *__restrict__ udst, double *__restrict__ vdst,
                               double *__restrict__ sdst)
{
    __shared__ double ru[128], rv[128];
    const ColJob j = jobs[blockIdx.x];
    const double *u = usrc + j.us, *v = vsrc + j.vs;
    double su = 0.0, sv = 0.0;
    for (int i = threadIdx.x; i < j.len; i += blockDim.x) {
        su = fma(u[i], u[i], su);
        sv = fma(v[i], v[i], sv);
    }
    ru[threadIdx.x] = su;
    rv[threadIdx.x] = sv;
    __syncthreads();
    for (int k = blockDim.x / 2; k > 0; k >>= 1) {
        if (threadIdx.x < k) {
            ru[threadIdx.x] += ru[threadIdx.x + k];
            rv[threadIdx.x] += rv[threadIdx.x + k];
        }
        __syncthreads();
    }
    const double f1 = sqrt(ru[0]), f2 = sqrt(rv[0]);
    const double mm = j.mult >= 0 ? mult[j.mult] : 1.0;
    const double s = mm * f1 * f2;
    const bool keep = !(s < j.eps2);
    const double g1 = keep ? j.usign / f1 : 1.0, g2 = keep ? 1.0 / f2 : 1.0;
    for (int i = threadIdx.x; i < j.len; i += blockDim.x) {
        udst[j.ud + i] = keep ? u[i] * g1 : u[i];
        vdst[j.vd + i] = keep ? v[i] * g2 : v[i];
    }
    if (threadIdx.x == 0) sdst[j.sd] = keep ? s : 0.0;
}

// KS = K^-1 S padded with zero columns to `width` (ld r).
__global__ void build_ks_kernel(const CapItem *items, const double *kbase, const double *pool,
                                const long long *ksoff, int width, double *ks)
{
    const CapItem c = items[blockIdx.x];
    const int r = c.r1 + c.r2;
    const double *K = kbase + c.k;
    double *out = ks + ksoff[blockIdx.x];
    for (long long e = threadIdx.x; e < (long long)r * width; e += blockDim.x) {
        int i = (int)(e % r), j = (int)(e / r);
        double v = 0.0;
        if (j < r) {
            double s = j < c.r1 ? pool[c.s1 + j] : pool[c.s2 + j - c.r1];
            v = K[i + (long long)j * r] * s;
        }
        out[e] = v;
    }
}

// Leaves of B: leaf inverse plus every ancestor correction, parent first.
__global__ void leaf_assemble_kernel(const LeafJob *__restrict__ jobs,
                                     const AncTerm *__restrict__ terms,
                                     const double *__restrict__ leafinv,
                                     const double *__restrict__ gu, const double *__restrict__ gv,
                                     const double *__restrict__ d, int m,
                                     double *__restrict__ out)
{
    const LeafJob L = jobs[blockIdx.x];
    const long long cnt = (long long)L.b * L.b;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        int i = (int)(e % L.b), jj = (int)(e / L.b);
        double acc = leafinv[L.src + e];
        for (int q = 0; q < L.count; ++q) {
            const AncTerm t = terms[L.first + q];
            double s = 0.0;
            for (int k = 0; k < t.k; ++k)
                s = fma(gu[t.goff + L.row0 + i + (long long)k * m] * d[t.doff + k],
                        gv[t.goff + L.row0 + jj + (long long)k * m], s);
            acc += s;
        }
        out[L.dst + e] = acc;
    }
}

static long long al32(long long x) { return (x + 31) & ~31LL; }

template <class T>
static int vec_to_dev(const std::vector<T> &v, T **dst)
{
    DG_ALLOC(dst, std::max<size_t>(v.size(), 1) * sizeof(T));
    if (!v.empty()) DG_CUDA(cudaMemcpy(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
    return 0;
}

struct DevBuf {
    std::vector<void *> ptrs;
    ~DevBuf()
    {
        for (void *p : ptrs) cudaFree(p);
    }
    int alloc(double **p, long long n)
    {
        cudaError_t e = dev_malloc((void **)p, std::max<long long>(n, 1) * sizeof(double));
        if (e != cudaSuccess) return fail(DPLR_GPU_ENOMEM, "geinv: cannot allocate %lld doubles", n);
        ptrs.push_back(*p);
        return 0;
    }
    template <class T> int upload(const std::vector<T> &v, T **p)
    {
        int rc = vec_to_dev(v, p);
        if (!rc) ptrs.push_back((void *)*p);
        return rc;
    }
};

// Everything the host replay needs about the device results.
struct InvResult {
    std::vector<long long> bu, bv, bs;   // per low-rank block: staging offsets
    std::vector<int> own;                // own columns per block (0 for stale nodes)
    std::vector<std::vector<int>> groups;   // per block: appended group sizes, parent first
    std::vector<long long> leafdst;      // per leaf: staging offset
    std::vector<double> hu, hv, hs, hleaf;   // host copies of the staging buffers
};

// Device computation of all values of B.
static int compute_inverse(Plan *p, Fact *F, double eps, cudaStream_t st, InvResult &R)
{
    const int m = p->m;
    const int nlev = (int)F->lv.size();
    DevBuf mem;
    int rc;

    // Thresholds eps2 per node: eps divided by 2 (children are leaves) or 4
    // at every node from the root down (src/dplrinv.c:154-171).
    std::vector<double> eps2(p->nodes.size());
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        const HDesc &H = p->nodes[nd];
        double in = H.parent < 0 ? eps : eps2[H.parent];
        eps2[nd] = H.nw < 0 ? in / 2.0 : in / 4.0;
    }

    // P_l = -Z_l K^-1 S per level.
    std::vector<long long> poff(nlev), goff(nlev);
    std::vector<int> w2(nlev, 0), wg(nlev, 0);
    long long ptot = 0, gtot = 0;
    for (int l = 0; l < nlev; ++l) {
        for (int nd : F->lv[l].nodes) {
            int r1 = p->lr[p->nodes[nd].ne].rank, r2 = p->lr[p->nodes[nd].sw].rank;
            w2[l] = std::max(w2[l], r1 + r2);
            wg[l] = std::max(wg[l], std::max(r1, r2));
        }
        poff[l] = ptot;
        ptot += al32((long long)m * w2[l]);
        goff[l] = gtot;
        gtot += al32((long long)m * wg[l]);
    }
    double *P = nullptr, *KS = nullptr, *Gu = nullptr, *Gv = nullptr, *D = nullptr;
    if ((rc = mem.alloc(&P, ptot)) || (rc = mem.alloc(&Gu, gtot)) || (rc = mem.alloc(&Gv, gtot)))
        return rc;
    std::vector<long long> doff(p->nodes.size());
    long long dtot = 0;
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        doff[nd] = dtot;
        dtot += p->lr[p->nodes[nd].ne].rank + p->lr[p->nodes[nd].sw].rank;
    }
    if ((rc = mem.alloc(&D, dtot))) return rc;

    const int TR = tile_rows_for(p);
    for (int l = 0; l < nlev; ++l) {
        const LevelOps &L = F->lv[l];
        if (L.n.caps.empty()) continue;
        std::vector<long long> ksoff;
        long long kstot = 0;
        for (const CapItem &c : L.n.caps) {
            ksoff.push_back(kstot);
            kstot += al32((long long)(c.r1 + c.r2) * w2[l]);
        }
        if ((rc = mem.alloc(&KS, kstot))) return rc;
        long long *d_ksoff = nullptr;
        if ((rc = mem.upload(ksoff, &d_ksoff))) return rc;
        build_ks_kernel<<<(unsigned)L.n.caps.size(), 256, 0, st>>>(L.n.d_caps, F->kpool, p->pool,
                                                                   d_ksoff, w2[l], KS);
        note_launch();
        DG_CUDA(cudaGetLastError());
        // Expand schedule: tiles of each node's nw rows use Z_l rows with
        // KS rows 0..r1, tiles of its se rows use KS rows r1..r.
        Schedule S;
        S.tile_rows = TR;
        size_t ci = 0;
        for (int nd : L.nodes) {
            const HDesc &H = p->nodes[nd];
            const int r1 = p->lr[H.ne].rank, r2 = p->lr[H.sw].rank, r = r1 + r2;
            if (r == 0) continue;
            const long long ks = ksoff[ci++];
            const int h = H.m / 2;
            for (int side = 0; side < 2; ++side) {
                int k = side == 0 ? r1 : r2;
                int row0 = H.row0 + side * h;
                for (int t0 = row0; t0 < row0 + h; t0 += TR) {
                    TileTerm tt;
                    tt.a = F->zoff[l] + t0;
                    tt.lda = m;
                    tt.K = k;
                    tt.trans_a = 0;
                    tt.src = 2;
                    tt.b = ks + (side == 0 ? 0 : r1);
                    tt.ldb = r;
                    tt.x_row0 = 0;
                    S.tile_row0.push_back(t0);
                    S.tile_begin.push_back((int)S.terms.size());
                    if (k > 0) S.terms.push_back(tt);
                }
            }
        }
        S.tile_begin.push_back((int)S.terms.size());
        long long dummy = 0;
        if ((rc = upload_schedule(S, &dummy))) return rc;
        rc = run_expand(S, F->zpool, KS, nullptr, 0, P + poff[l], m, w2[l], -1.0, 0.0, st);
        cudaError_t e = cudaStreamSynchronize(st);
        free_schedule(S);
        if (rc) return rc;
        if (e != cudaSuccess) return fail(DPLR_GPU_ECUDA, "geinv: %s", cudaGetErrorString(e));
    }

    // Correction generators of every node, normalised with the node's eps2
    // (src/dplrinv.c:376-423): nw side  (-u1 Y12, v2),  se side (-u2 Y21, v1).
    std::vector<ColJob> gjobs;
    for (int l = 0; l < nlev; ++l)
        for (int nd : F->lv[l].nodes) {
            const HDesc &H = p->nodes[nd];
            const int r1 = p->lr[H.ne].rank, r2 = p->lr[H.sw].rank, h = H.m / 2;
            const int c1 = H.row0, c2 = H.row0 + h;
            for (int i = 0; i < r2; ++i) {   // nw side, d at doff + i
                ColJob j;
                j.us = poff[l] + c1 + (long long)(r1 + i) * m;
                j.vs = F->zoff[l] + c1 + (long long)i * m;
                j.ud = j.vd = goff[l] + c1 + (long long)i * m;
                j.sd = doff[nd] + i;
                j.mult = -1;
                j.eps2 = eps2[nd];
                j.usign = 1.0;
                j.len = h;
                gjobs.push_back(j);
            }
            for (int i = 0; i < r1; ++i) {   // se side, d at doff + r2 + i
                ColJob j;
                j.us = poff[l] + c2 + (long long)i * m;
                j.vs = F->zoff[l] + c2 + (long long)i * m;
                j.ud = j.vd = goff[l] + c2 + (long long)i * m;
                j.sd = doff[nd] + r2 + i;
                j.mult = -1;
                j.eps2 = eps2[nd];
                j.usign = 1.0;
                j.len = h;
                gjobs.push_back(j);
            }
        }
    if (!gjobs.empty()) {
        ColJob *d_g = nullptr;
        if ((rc = mem.upload(gjobs, &d_g))) return rc;
        colpair_kernel<<<(unsigned)gjobs.size(), 128, 0, st>>>(d_g, P, F->ztpool, nullptr, Gu, Gv, D);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }

    // Columns of every low-rank block of B: own columns, then one group per
    // ancestor (parent first) on the side of the ancestor holding the block.
    const size_t nb = p->lr.size();
    R.bu.assign(nb, 0);
    R.bv.assign(nb, 0);
    R.bs.assign(nb, 0);
    R.own.assign(nb, 0);
    R.groups.assign(nb, {});
    std::vector<ColJob> own, app;
    long long btot = 0, stot = 0;
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        const HDesc &H = p->nodes[nd];
        const int l = H.level, h = H.m / 2;
        const int r1 = p->lr[H.ne].rank, r2 = p->lr[H.sw].rank;
        const bool stale = r1 == 0 && r2 == 0;
        for (int s = 0; s < 2; ++s) {
            const int b = s == 0 ? H.ne : H.sw;
            const int urow = s == 0 ? H.row0 : H.row0 + h;   // rows of the block
            const int vrow = s == 0 ? H.row0 + h : H.row0;   // columns of the block
            int ncols = stale ? 0 : (s == 0 ? r1 : r2);
            R.own[b] = ncols;
            std::vector<int> grp;
            for (int a = H.parent, child = (int)nd; a >= 0; child = a, a = p->nodes[a].parent) {
                const HDesc &A = p->nodes[a];
                const bool nwside = H.row0 < A.row0 + A.m / 2;
                const int k = nwside ? p->lr[A.sw].rank : p->lr[A.ne].rank;
                if (k > 0) grp.push_back(k);
                ncols += k;
                (void)child;
            }
            R.groups[b] = grp;
            R.bu[b] = btot;
            R.bv[b] = btot;
            btot += al32((long long)h * ncols);
            R.bs[b] = stot;
            stot += ncols;
            int col = 0;
            for (int i = 0; i < R.own[b]; ++i, ++col) {
                ColJob j;
                j.us = poff[l] + urow + (long long)(s == 0 ? i : r1 + i) * m;
                j.vs = F->zoff[l] + vrow + (long long)i * m;
                j.ud = R.bu[b] + (long long)col * h;
                j.vd = R.bv[b] + (long long)col * h;
                j.sd = R.bs[b] + col;
                j.mult = -1;
                j.eps2 = eps2[nd];
                j.usign = 1.0;
                j.len = h;
                own.push_back(j);
            }
            for (int a = H.parent; a >= 0; a = p->nodes[a].parent) {
                const HDesc &A = p->nodes[a];
                const bool nwside = H.row0 < A.row0 + A.m / 2;
                const int ar1 = p->lr[A.ne].rank, ar2 = p->lr[A.sw].rank;
                const int k = nwside ? ar2 : ar1;
                const long long d0 = doff[a] + (nwside ? 0 : ar2);
                for (int i = 0; i < k; ++i, ++col) {
                    ColJob j;
                    j.us = goff[A.level] + urow + (long long)i * m;
                    j.vs = goff[A.level] + vrow + (long long)i * m;
                    j.ud = R.bu[b] + (long long)col * h;
                    j.vd = R.bv[b] + (long long)col * h;
                    j.sd = R.bs[b] + col;
                    j.mult = d0 + i;
                    j.eps2 = eps2[nd];
                    j.usign = 1.0;
                    j.len = h;
                    app.push_back(j);
                }
            }
        }
    }
    double *BU = nullptr, *BV = nullptr, *BS = nullptr;
    if ((rc = mem.alloc(&BU, btot)) || (rc = mem.alloc(&BV, btot)) || (rc = mem.alloc(&BS, stot)))
        return rc;
    if (!own.empty()) {
        ColJob *d_o = nullptr;
        if ((rc = mem.upload(own, &d_o))) return rc;
        colpair_kernel<<<(unsigned)own.size(), 128, 0, st>>>(d_o, P, F->ztpool, nullptr, BU, BV, BS);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    if (!app.empty()) {
        ColJob *d_a = nullptr;
        if ((rc = mem.upload(app, &d_a))) return rc;
        colpair_kernel<<<(unsigned)app.size(), 128, 0, st>>>(d_a, Gu, Gv, D, BU, BV, BS);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }

    // Leaves.
    std::vector<LeafJob> ljobs;
    std::vector<AncTerm> terms;
    R.leafdst.clear();
    long long ltot = 0;
    // parent of each leaf: the H node whose nw/se is ~leaf
    std::vector<int> leaf_parent(p->leaves.size(), -1);
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        if (p->nodes[nd].nw < 0) leaf_parent[~p->nodes[nd].nw] = (int)nd;
        if (p->nodes[nd].se < 0) leaf_parent[~p->nodes[nd].se] = (int)nd;
    }
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        const LeafDesc &Lf = p->leaves[i];
        LeafJob j;
        j.src = F->leafoff[i];
        j.dst = ltot;
        j.row0 = Lf.row0;
        j.b = Lf.b;
        j.first = (int)terms.size();
        for (int a = leaf_parent[i]; a >= 0; a = p->nodes[a].parent) {
            const HDesc &A = p->nodes[a];
            const bool nwside = Lf.row0 < A.row0 + A.m / 2;
            const int ar1 = p->lr[A.ne].rank, ar2 = p->lr[A.sw].rank;
            AncTerm t;
            t.k = nwside ? ar2 : ar1;
            t.goff = goff[A.level];
            t.doff = doff[a] + (nwside ? 0 : ar2);
            if (t.k > 0) terms.push_back(t);
        }
        j.count = (int)terms.size() - j.first;
        R.leafdst.push_back(ltot);
        ltot += al32((long long)Lf.b * Lf.b);
        ljobs.push_back(j);
    }
    double *LB = nullptr;
    if ((rc = mem.alloc(&LB, ltot))) return rc;
    if (!ljobs.empty()) {
        LeafJob *d_l = nullptr;
        AncTerm *d_t = nullptr;
        if ((rc = mem.upload(ljobs, &d_l)) || (rc = mem.upload(terms, &d_t))) return rc;
        leaf_assemble_kernel<<<(unsigned)ljobs.size(), 256, 0, st>>>(d_l, d_t, F->leafinv, Gu, Gv, D,
                                                                     m, LB);
        note_launch();
        DG_CUDA(cudaGetLastError());
    }
    DG_CUDA(cudaStreamSynchronize(st));
    R.hu.resize(std::max<long long>(btot, 1));
    R.hv.resize(std::max<long long>(btot, 1));
    R.hs.resize(std::max<long long>(stot, 1));
    R.hleaf.resize(std::max<long long>(ltot, 1));
    DG_CUDA(cudaMemcpy(R.hu.data(), BU, btot * sizeof(double), cudaMemcpyDeviceToHost));
    DG_CUDA(cudaMemcpy(R.hv.data(), BV, btot * sizeof(double), cudaMemcpyDeviceToHost));
    DG_CUDA(cudaMemcpy(R.hs.data(), BS, stot * sizeof(double), cudaMemcpyDeviceToHost));
    DG_CUDA(cudaMemcpy(R.hleaf.data(), LB, ltot * sizeof(double), cudaMemcpyDeviceToHost));
    return 0;
}

// Host replay of DPLR's structural steps on B, in DPLR's order, copying
// the computed values in (src/dplrinv.c:124-221, src/dplrprk.c:99-191).
struct Replay {
    Plan *p;
    const InvResult &R;
    int node_i = 0, leaf_i = 0;
    std::vector<DPlrMtx *> blocks;     // B's low-rank blocks in plan order

    void walk(const DPlrMtx *A, DPlrMtx *B)
    {
        if (A->type == PLR_DMTX) {
            const int li = leaf_i++;
            const int m = A->size;
            if (B->type != PLR_DMTX || B->size != m) {
                dplrclr(B);
                dplrinid(m, B);
            }
            memcpy(B->dd.d, R.hleaf.data() + R.leafdst[li], sizeof(double) * m * m);
            return;
        }
        const int nd = node_i++;
        const int m = A->size, h = m / 2;
        if (B->type != PLR_HMTX || B->size != m) {
            dplrclr(B);
            dplrinih(m, B);
        }
        const HDesc &H = p->nodes[nd];
        walk(A->dh.nw, B->dh.nw);
        walk(A->dh.se, B->dh.se);
        DPlrMtx *bl[2] = {B->dh.ne, B->dh.sw};
        const DPlrMtx *al[2] = {A->dh.ne, A->dh.sw};
        for (int s = 0; s < 2; ++s) {
            if (bl[s]->type != PLR_LRMTX || bl[s]->size != h) {
                dplrclr(bl[s]);
                dplrinilr(h, bl[s], al[s]->dlr.rank);
            }
            if (bl[s]->dlr.capacity < al[s]->dlr.rank) dplrresizelr(bl[s], al[s]->dlr.rank);
        }
        const int r1 = A->dh.ne->dlr.rank, r2 = A->dh.sw->dlr.rank;
        blocks[H.ne] = bl[0];
        blocks[H.sw] = bl[1];
        if (r1 == 0 && r2 == 0) return;
        for (int s = 0; s < 2; ++s) {
            const int b = s == 0 ? H.ne : H.sw;
            const int r = R.own[b];
            copy_cols(bl[s], b, 0, 0, r);
            bl[s]->dlr.rank = r;
        }
    }

    void copy_cols(DPlrMtx *L, int b, int src_col, int dst_col, int count)
    {
        if (count <= 0) return;
        const size_t n = (size_t)L->size;
        memcpy(L->dlr.u + n * dst_col, R.hu.data() + R.bu[b] + n * src_col, sizeof(double) * n * count);
        memcpy(L->dlr.v + n * dst_col, R.hv.data() + R.bv[b] + n * src_col, sizeof(double) * n * count);
        memcpy(L->dlr.sig + dst_col, R.hs.data() + R.bs[b] + src_col, sizeof(double) * count);
    }

    // dplrgeprk's appends, block by block, parent first: grow capacity the
    // way dplrresizelr does, then place the group after the live columns.
    void appends()
    {
        for (size_t b = 0; b < blocks.size(); ++b) {
            DPlrMtx *L = blocks[b];
            int src = R.own[b];
            for (int k : R.groups[b]) {
                const int r = L->dlr.rank;
                if (L->dlr.capacity < r + k) dplrresizelr(L, r + k);
                copy_cols(L, (int)b, src, r, k);
                L->dlr.rank = r + k;
                src += k;
            }
        }
    }
};

}  // namespace dg

using namespace dg;

extern "C" void dplrgeinv(int m, DPlrMtx *A, DPlrMtx *B, double eps, int *info)
{
    dg::NvtxRange nvtx_("dplrgeinv");
    const char *fn = "dplrgeinv";
    if (m < 0) {
        fprintf(stderr, "%s: invalid matrix size: %d\n", fn, m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "%s: invalid A type\n", fn);
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "%s: invalid A size\n", fn);
        return;
    }
    *info = -1;
    if (validate_tree(m, A, fn)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    Plan *p = nullptr;
    if (plan_build(m, A, 0, &p)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    int rc = factor_build(p, DPLR_GPU_FACTOR_TRANSPOSED, 0);
    if (rc) {
        Fact *F = (Fact *)p->fact;
        if (rc == DPLR_GPU_ESINGULAR && F && F->sing_info > 0) *info = F->sing_info;
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        plan_free(p);
        return;
    }
    InvResult R;
    rc = compute_inverse(p, (Fact *)p->fact, eps, 0, R);
    if (rc) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        plan_free(p);
        return;
    }
    Replay rp{p, R};
    rp.blocks.assign(p->lr.size(), nullptr);
    rp.walk(A, B);
    rp.appends();
    plan_free(p);
    *info = 0;
    recompress_after(m, B);
}

// ---------------------------------------------------------------- geprk
namespace dg {

// Leaf update of dplrgeprk: D += alpha * (u[rows] diag(s)) v[rows]^T.
__global__ void leaf_rank_update_kernel(const LeafJob *__restrict__ jobs,
                                        const double *__restrict__ pool,
                                        const double *__restrict__ U, const double *__restrict__ V,
                                        const double *__restrict__ s, int k, int m, double alpha,
                                        double *__restrict__ out)
{
    const LeafJob L = jobs[blockIdx.x];
    const long long cnt = (long long)L.b * L.b;
    for (long long e = threadIdx.x; e < cnt; e += blockDim.x) {
        int i = (int)(e % L.b), jj = (int)(e / L.b);
        double acc = 0.0;
        for (int q = 0; q < k; ++q)
            acc = fma(U[L.row0 + i + (long long)q * m] * s[q], V[L.row0 + jj + (long long)q * m], acc);
        out[L.dst + e] = fma(alpha, acc, pool[L.src + e]);
    }
}

}  // namespace dg

// A += alpha * u diag(s) v^T (DPLR src/dplrprk.c:21-199): every low-rank
// block gets the k column pairs restricted to its rows and columns,
// normalised (sig = |alpha| s_i |u_i| |v_i|, zeroed below the node's
// threshold, sign of alpha folded into u); every leaf gets the dense
// rank-k update.  Norms, scaling and leaf products run on the GPU; the host
// grows capacities like dplrresizelr and stores the results.
extern "C" void dplrgeprk(int m, int k, double *alpha, double *u, int ldu, double *v, int ldv,
                          double *s, int incs, DPlrMtx *A, double eps)
{
    dg::NvtxRange nvtx_("dplrgeprk");
    const char *fn = "dplrgeprk";
    if (m < 0) {
        fprintf(stderr, "%s: invalid matrix size %d\n", fn, m);
        return;
    }
    if (A->type != PLR_DMTX && A->type != PLR_HMTX) {
        fprintf(stderr, "%s: invalid A type\n", fn);
        return;
    }
    if (A->size != m) {
        fprintf(stderr, "%s: invalid A size\n", fn);
        return;
    }
    if (ldu < m || ldv < m) {
        fprintf(stderr, "%s: invalid leading dimensions\n", fn);
        return;
    }
    if (*alpha == 0.0 || k == 0) return;
    if (k < 0 || incs < 1) {
        fprintf(stderr, "%s: invalid k or incs\n", fn);
        return;
    }
    if (validate_tree(m, A, fn)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    Plan *p = nullptr;
    if (plan_build(m, A, 0, &p)) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        return;
    }
    auto bail = [&](void) {
        fprintf(stderr, "%s: %s\n", fn, dplr_gpu_last_error());
        plan_free(p);
    };
    DevBuf mem;
    double *U = nullptr, *V = nullptr, *S = nullptr;
    if (mem.alloc(&U, (long long)m * k) || mem.alloc(&V, (long long)m * k) || mem.alloc(&S, k))
        return bail();
    std::vector<double> hs(k);
    for (int i = 0; i < k; ++i) hs[i] = s[(size_t)i * incs];
    if (cudaMemcpy2D(U, sizeof(double) * m, u, sizeof(double) * ldu, sizeof(double) * m, k,
                     cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy2D(V, sizeof(double) * m, v, sizeof(double) * ldv, sizeof(double) * m, k,
                     cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(S, hs.data(), sizeof(double) * k, cudaMemcpyHostToDevice) != cudaSuccess) {
        fail(DPLR_GPU_ECUDA, "upload of u, v, s failed");
        return bail();
    }
    const double mag = fabs(*alpha);
    std::vector<double> mult(k);
    for (int i = 0; i < k; ++i) mult[i] = mag * hs[i];
    double *M = nullptr;
    if (mem.alloc(&M, k) ||
        cudaMemcpy(M, mult.data(), sizeof(double) * k, cudaMemcpyHostToDevice) != cudaSuccess)
        return bail();

    // Thresholds: eps/2 or eps/4 at each node, compounded from the root.
    std::vector<double> eps2(p->nodes.size());
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        const HDesc &H = p->nodes[nd];
        double in = H.parent < 0 ? eps : eps2[H.parent];
        eps2[nd] = H.nw < 0 ? in / 2.0 : in / 4.0;
    }
    std::vector<ColJob> jobs;
    std::vector<long long> boff(p->lr.size());
    long long btot = 0;
    for (size_t nd = 0; nd < p->nodes.size(); ++nd) {
        const HDesc &H = p->nodes[nd];
        const int h = H.m / 2;
        for (int side = 0; side < 2; ++side) {
            const int b = side == 0 ? H.ne : H.sw;
            const int urow = side == 0 ? H.row0 : H.row0 + h;
            const int vrow = side == 0 ? H.row0 + h : H.row0;
            boff[b] = btot;
            for (int i = 0; i < k; ++i) {
                ColJob j;
                j.us = urow + (long long)i * m;
                j.vs = vrow + (long long)i * m;
                j.ud = j.vd = btot + (long long)i * h;
                j.sd = 0;   // set below
                j.mult = i;
                j.eps2 = eps2[nd];
                j.usign = *alpha > 0.0 ? 1.0 : -1.0;
                j.len = h;
                jobs.push_back(j);
            }
            btot += al32((long long)h * k);
        }
    }
    std::vector<long long> soff(p->lr.size());
    for (size_t b = 0; b < p->lr.size(); ++b) soff[b] = (long long)b * k;
    for (size_t q = 0; q < jobs.size(); ++q) jobs[q].sd = (long long)q;   // one sig per job
    double *BU = nullptr, *BV = nullptr, *BS = nullptr, *LB = nullptr;
    if (mem.alloc(&BU, btot) || mem.alloc(&BV, btot) || mem.alloc(&BS, (long long)jobs.size()))
        return bail();
    if (!jobs.empty()) {
        ColJob *d_j = nullptr;
        if (mem.upload(jobs, &d_j)) return bail();
        colpair_kernel<<<(unsigned)jobs.size(), 128>>>(d_j, U, V, M, BU, BV, BS);
        note_launch();
        if (cudaGetLastError() != cudaSuccess) {
            fail(DPLR_GPU_ECUDA, "column normalisation launch failed");
            return bail();
        }
    }
    std::vector<LeafJob> ljobs;
    long long ltot = 0;
    for (size_t i = 0; i < p->leaves.size(); ++i) {
        LeafJob j;
        j.src = p->leaves[i].d;
        j.dst = ltot;
        j.row0 = p->leaves[i].row0;
        j.b = p->leaves[i].b;
        j.first = j.count = 0;
        ljobs.push_back(j);
        ltot += al32((long long)j.b * j.b);
    }
    if (mem.alloc(&LB, ltot)) return bail();
    if (!ljobs.empty()) {
        LeafJob *d_l = nullptr;
        if (mem.upload(ljobs, &d_l)) return bail();
        leaf_rank_update_kernel<<<(unsigned)ljobs.size(), 256>>>(d_l, p->pool, U, V, S, k, m, *alpha,
                                                                 LB);
        note_launch();
    }
    std::vector<double> hu(std::max<long long>(btot, 1)), hv(std::max<long long>(btot, 1)),
        hsig(std::max<size_t>(jobs.size(), 1)), hl(std::max<long long>(ltot, 1));
    if (cudaDeviceSynchronize() != cudaSuccess ||
        cudaMemcpy(hu.data(), BU, btot * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hv.data(), BV, btot * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hsig.data(), BS, jobs.size() * 8, cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(hl.data(), LB, ltot * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
        fail(DPLR_GPU_ECUDA, "rank update on the GPU failed: %s", cudaGetErrorString(cudaGetLastError()));
        return bail();
    }
    // Host: append in DPLR's order (ne then sw, pre-order), leaves in place.
    struct Walk {
        const Plan *p;
        int k;
        const std::vector<long long> &boff;
        const std::vector<double> &hu, &hv, &hsig, &hl;
        const std::vector<LeafJob> &lj;
        int node_i = 0, leaf_i = 0;
        void go(DPlrMtx *A)
        {
            if (A->type == PLR_DMTX) {
                const LeafJob &L = lj[leaf_i++];
                memcpy(A->dd.d, hl.data() + L.dst, sizeof(double) * L.b * L.b);
                return;
            }
            const HDesc &H = p->nodes[node_i++];
            DPlrMtx *bl[2] = {A->dh.ne, A->dh.sw};
            for (int s2 = 0; s2 < 2; ++s2) {
                const int b = s2 == 0 ? H.ne : H.sw;
                DPlrMtx *L = bl[s2];
                const int r = L->dlr.rank;
                if (L->dlr.capacity < r + k) dplrresizelr(L, r + k);
                const size_t n = (size_t)L->size;
                memcpy(L->dlr.u + n * r, hu.data() + boff[b], sizeof(double) * n * k);
                memcpy(L->dlr.v + n * r, hv.data() + boff[b], sizeof(double) * n * k);
                memcpy(L->dlr.sig + r, hsig.data() + (size_t)b * k, sizeof(double) * k);
                L->dlr.rank = r + k;
            }
            go(A->dh.nw);
            go(A->dh.se);
        }
    } w{p, k, boff, hu, hv, hsig, hl, ljobs};
    w.go(A);
    plan_free(p);
    recompress_after(m, A);
}
