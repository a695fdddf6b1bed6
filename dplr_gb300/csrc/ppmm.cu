// ppmm.cu -- dplrgeppmm on the GPU: C := alpha op(A) op(B) + beta C for PLR
// matrices A, B, C of one structure (DPLR src/dplrppmm.c:998 with dplrplmm
// :185, dplrlpmm :334, dplrgellmm :26 and dplrgeprk, src/dplrprk.c:21).
//
// DPLR recurses: dense leaves are multiplied (dgemm); at an H node X with
// op(M).ne = M.ne or M.sw^T and op(M).sw = M.sw or M.ne^T,
//   C.ne gets [beta C.ne | op(A).nw op(B).ne | op(A).ne op(B).se],
//   C.sw gets [beta C.sw | op(A).sw op(B).nw | op(A).se op(B).sw],
// each product of a subtree P and a low-rank block L (or L and P) being
// op(P) L.u (op(P)^T L.v) normalised column by column with the threshold
// eps/4^(depth+1); then C.nw and C.se recurse, and the products
// op(A).ne op(B).sw and op(A).sw op(B).ne of two low-rank blocks (rank
// min(r1, r2)) are added to them by dplrgeprk, which appends the
// restricted, normalised columns to every low-rank block below and adds
// them to the leaves.  Nothing is recompressed, so every column of the
// result and its place are known in advance:
//   block of node Y = [beta part | own products | ancestor terms, parent
//   first], leaf = alpha op(A) op(B) + beta C + ancestor terms.
//
// The GPU computes all of them at once from device copies of A, B and C:
//   1. one batched FP64 GEMM launch multiplies every leaf;
//   2. per depth d, one apply of the block-diagonal part of op(A) made of
//      its depth-(d+1) subtrees (the apply kernels with a depth-filtered
//      schedule) to a stack of every node's op(B).ne / op(B).sw u-factors,
//      and one of op(B)^T to the op(A) v-factors: all products of that depth;
//   3. two batched GEMM launches form the low-rank x low-rank terms;
//   4. one launch normalises the terms' computed sides, one builds every
//      column of every block of C (norms, threshold, scaled or raw copy);
//   5. one batched GEMM launch per ancestor distance adds the terms to the
//      leaves.
// The host replays DPLR's capacity growth (dplrresizelr per append, in
// order) on C and stores the columns, so ranks, capacities and column
// order are DPLR's.
#include "internal.cuh"
#include "gemm.cuh"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <thread>
#include <vector>

namespace dg {

namespace {

// ------------------------------------------------------------ kernels --

// One column pair of C (or one side of a term), built from its sources.
enum ColMode { kOld = 0, kNormU = 1, kNormV = 2, kNormUV = 3 };

struct ColJob {
    const double *su, *sv;   // source columns (n doubles each), may be null
    double *du, *dv;         // destinations, may be null (du == su allowed)
    double *dsig;            // destination of the singular value
    const double *ss;        // singular value of the generating column
    double sm;               // its multiplier
    double thr;              // threshold of the normalising modes
    double g;                // kOld: factor of u; kNormUV: sign folded into u
    int n, mode;
};

__device__ double block_sum(double v, double *red)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    __syncthreads();
    if (l == 0) red[w] = v;
    __syncthreads();
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
    return s;
}

__global__ void __launch_bounds__(128) col_kernel(const ColJob *__restrict__ jobs)
{
    __shared__ double red[4];
    const ColJob J = jobs[blockIdx.x];
    const double s = J.sm * J.ss[0];
    if (J.mode == kOld) {
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) {
            J.du[i] = J.g * J.su[i];
            J.dv[i] = J.sv[i];
        }
        if (threadIdx.x == 0) J.dsig[0] = s;
        return;
    }
    double qu = 0.0, qv = 0.0;
    if (J.mode != kNormV)
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) qu = fma(J.su[i], J.su[i], qu);
    if (J.mode != kNormU)
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) qv = fma(J.sv[i], J.sv[i], qv);
    const double fu = J.mode != kNormV ? sqrt(block_sum(qu, red)) : 1.0;
    const double fv = J.mode != kNormU ? sqrt(block_sum(qv, red)) : 1.0;
    double val;
    if (J.mode == kNormU) val = fu * s;
    else if (J.mode == kNormV) val = fv * s;
    else val = s * fu * fv;
    const bool keep = !(val < J.thr);
    const double cu = !keep || J.mode == kNormV ? 1.0 : (J.mode == kNormUV ? J.g * (1.0 / fu) : 1.0 / fu);
    const double cv = !keep || J.mode == kNormU ? 1.0 : 1.0 / fv;
    __syncthreads();   // every norm read precedes the in-place writes
    if (J.du)
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) J.du[i] = cu == 1.0 ? J.su[i] : J.su[i] * cu;
    if (J.dv)
        for (int i = threadIdx.x; i < J.n; i += blockDim.x) J.dv[i] = cv == 1.0 ? J.sv[i] : J.sv[i] * cv;
    if (threadIdx.x == 0) J.dsig[0] = keep ? val : 0.0;
}

// Strided block copies (rows x cols), one CTA per (job, column).
struct CopyJob {
    const double *src;
    double *dst;
    int lds, ldd, rows;
};

__global__ void copy_kernel(const CopyJob *__restrict__ jobs, const int2 *__restrict__ items)
{
    const int2 it = items[blockIdx.x];
    const CopyJob J = jobs[it.x];
    const double *s = J.src + (long long)it.y * J.lds;
    double *d = J.dst + (long long)it.y * J.ldd;
    for (int i = threadIdx.x; i < J.rows; i += blockDim.x) d[i] = s[i];
}

// ---------------------------------------------------------- host side --

// Device memory of one call, stream-ordered (cudaMallocAsync), released
// after the call's work.
struct Arena {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Arena(cudaStream_t s) : st(s) {}
    ~Arena()
    {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    template <class T> int alloc(T **p, long long n)
    {
        if (cudaMallocAsync((void **)p, (size_t)std::max<long long>(n, 1) * sizeof(T), st) != cudaSuccess)
            return fail(DPLR_GPU_ENOMEM, "dplrgeppmm: cannot allocate %lld bytes", n * (long long)sizeof(T));
        ptrs.push_back(*p);
        return 0;
    }
    template <class T> int upload(const std::vector<T> &v, T **p)
    {
        int rc = alloc(p, (long long)v.size());
        if (rc) return rc;
        if (!v.empty()) DG_CUDA(cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
        return 0;
    }
};

int launch_gemms(Arena &ar, const std::vector<GemmJob> &jobs, cudaStream_t st)
{
    if (jobs.empty()) return 0;
    std::vector<GemmTile> tiles;
    std::vector<GemmRed> reds;
    long long ptot = 0;
    plan_gemm_tiles(jobs, tiles, reds, ptot);
    if (tiles.empty()) return 0;
    GemmJob *dj;
    GemmTile *dt;
    GemmRed *dr = nullptr;
    double *part = nullptr;
    int rc;
    if ((rc = ar.upload(jobs, &dj)) || (rc = ar.upload(tiles, &dt))) return rc;
    if (!reds.empty() && ((rc = ar.upload(reds, &dr)) || (rc = ar.alloc(&part, ptot)))) return rc;
    run_gemm_tables(dj, dt, tiles.size(), dr, reds.size(), part, st);
    note_launches((long long)((tiles.size() + (1u << 30) - 1) >> 30) + (reds.empty() ? 0 : 1));
    DG_CUDA(cudaGetLastError());
    return 0;
}

int launch_cols(Arena &ar, const std::vector<ColJob> &jobs, cudaStream_t st)
{
    if (jobs.empty()) return 0;
    ColJob *dj;
    int rc = ar.upload(jobs, &dj);
    if (rc) return rc;
    for (size_t b0 = 0; b0 < jobs.size(); b0 += 1u << 30) {
        const unsigned nb = (unsigned)std::min<size_t>(jobs.size() - b0, 1u << 30);
        col_kernel<<<nb, 128, 0, st>>>(dj + b0);
        note_launch();
    }
    DG_CUDA(cudaGetLastError());
    return 0;
}

int launch_copies(Arena &ar, const std::vector<CopyJob> &jobs, const std::vector<int> &cols, cudaStream_t st)
{
    std::vector<int2> items;
    for (int j = 0; j < (int)jobs.size(); ++j)
        for (int c = 0; c < cols[j]; ++c) items.push_back(make_int2(j, c));
    if (items.empty()) return 0;
    CopyJob *dj;
    int2 *di;
    int rc;
    if ((rc = ar.upload(jobs, &dj)) || (rc = ar.upload(items, &di))) return rc;
    copy_kernel<<<(unsigned)items.size(), 256, 0, st>>>(dj, di);
    note_launch();
    DG_CUDA(cudaGetLastError());
    return 0;
}

// Pinned host staging of the result, kept between calls and grown on
// demand (dplr_gpu_release_staging frees it).
struct Staging {
    std::mutex mu;
    double *p = nullptr;
    size_t n = 0;
};

Staging &staging()
{
    static Staging s;
    return s;
}

// op(M)'s view of a low-rank block: u-side, v-side, singular values.
struct View {
    const double *U, *V, *S;
    int r, n;
};

View view_of(const Plan *p, int b, bool t)
{
    const LRDesc &L = p->lr[b];
    return View{p->pool + (t ? L.v : L.u), p->pool + (t ? L.u : L.v), p->pool + L.sig, L.rank, L.n};
}
View op_ne(const Plan *p, const HDesc &H, bool t) { return t ? view_of(p, H.sw, true) : view_of(p, H.ne, false); }
View op_sw(const Plan *p, const HDesc &H, bool t) { return t ? view_of(p, H.ne, true) : view_of(p, H.sw, false); }

// Low-rank x low-rank term of one H node (dplrgellmm with beta = 0),
// added by dplrgeprk to the diagonal child `target` (HDesc index, or
// ~leaf).
struct Term {
    const double *u, *v;   // h x k, ld h
    double *s;             // k
    int k = 0, h = 0, row0 = 0;
    int target = 0;
    double eps = 0;        // threshold handed to dplrgeprk
};

// One segment of a block of C: `count` columns built by ColJobs.
struct Segment {
    int kind;              // 0 beta part, 1 plmm, 2 lpmm, 3 term
    int count;
    int term;              // kind 3
};

void collect(DPlrMtx *T, std::vector<DPlrMtx *> &lrs, std::vector<DPlrMtx *> &leaves)
{
    if (T->type == PLR_DMTX) {
        leaves.push_back(T);
        return;
    }
    lrs.push_back(T->dh.ne);
    lrs.push_back(T->dh.sw);
    collect(T->dh.nw, lrs, leaves);
    collect(T->dh.se, lrs, leaves);
}

int same_structure(const DPlrMtx *a, const DPlrMtx *b, const DPlrMtx *c, const char *fn)
{
    if (a->type != b->type || b->type != c->type) return fail(DPLR_GPU_EINVAL, "%s: A, B and C type do not match", fn);
    if (a->type != PLR_DMTX && a->type != PLR_HMTX) return fail(DPLR_GPU_EINVAL, "%s: invalid A, B or C type", fn);
    if (a->size != b->size || b->size != c->size) return fail(DPLR_GPU_EINVAL, "%s: invalid A, B or C size", fn);
    if (a->type == PLR_DMTX) return 0;
    int rc = same_structure(a->dh.nw, b->dh.nw, c->dh.nw, fn);
    return rc ? rc : same_structure(a->dh.se, b->dh.se, c->dh.se, fn);
}

struct PlanSet {
    Plan *a = nullptr, *b = nullptr, *c = nullptr;
    ~PlanSet()
    {
        if (a) plan_free(a);
        if (b) plan_free(b);
        if (c) plan_free(c);
    }
};

// Y = alpha * blockdiag_{depth >= lmin}(op(P)) X   (X, Y: m x nrhs, ld m)
int restricted_apply(Arena &ar, const Plan *p, int trans, int lmin, const double *X, double *Y, int nrhs,
                     double alpha, cudaStream_t st)
{
    Schedule S;
    build_schedule(p, trans, S, lmin);
    for (const PanelItem &it : S.items) S.max_len = std::max(S.max_len, it.len);
    for (const TileTerm &t : S.terms) S.has_row_major = S.has_row_major || t.trans_a;
    double *T = nullptr, *partials = nullptr;
    int rc;
    if ((rc = ar.upload(S.items, &S.d_items)) || (rc = ar.upload(S.reduces, &S.d_reduces)) ||
        (rc = ar.upload(S.tile_row0, &S.d_tile_row0)) || (rc = ar.upload(S.tile_begin, &S.d_tile_begin)) ||
        (rc = ar.upload(S.terms, &S.d_terms)))
        return rc;
    if ((rc = ar.alloc(&T, std::max<long long>(1, S.t_per_rhs * nrhs))) ||
        (rc = ar.alloc(&partials, std::max<long long>(1, S.partial_per_rhs * nrhs))))
        return rc;
    if ((rc = run_panel(S, p->pool, X, p->m, nrhs, partials, st))) return rc;
    if ((rc = run_reduce(S, p->pool, partials, nrhs, T, st))) return rc;
    return run_expand(S, p->pool, T, X, p->m, Y, p->m, nrhs, alpha, 0.0, st);
}

int geppmm_device(int ta, int tb, int m, double alpha, const DPlrMtx *A, const DPlrMtx *B, double beta, DPlrMtx *C,
                  double eps, cudaStream_t st)
{
    PlanSet ps;
    int rc;
    if ((rc = plan_build(m, A, st, &ps.a)) || (B != A && (rc = plan_build(m, B, st, &ps.b))) ||
        (rc = plan_build(m, C, st, &ps.c)))
        return rc;
    const Plan *pa = ps.a, *pb = B != A ? ps.b : ps.a, *pc = ps.c;
    const std::vector<HDesc> &nodes = pc->nodes;
    const int nH = (int)nodes.size(), nL = (int)pc->leaves.size();
    Arena ar(st);

    // thresholds of dplrppmm's recursion: eps/4 per level
    std::vector<double> e2(nH);
    for (int i = 0; i < nH; ++i) e2[i] = (nodes[i].parent < 0 ? eps : e2[nodes[i].parent]) / 4.0;

    // ---- the low-rank x low-rank terms (two per H node)
    std::vector<Term> terms;
    std::vector<int> term_of(2 * nH, -1);   // [2i]: term into C.nw of node i, [2i+1]: into C.se
    std::vector<GemmJob> g1, g2;
    std::vector<ColJob> tnorm;
    for (int i = 0; i < nH; ++i) {
        const HDesc &H = nodes[i];
        for (int side = 0; side < 2; ++side) {
            // nw: op(A).ne x op(B).sw ; se: op(A).sw x op(B).ne
            const View L1 = side == 0 ? op_ne(pa, H, ta) : op_sw(pa, H, ta);
            const View L2 = side == 0 ? op_sw(pb, H, tb) : op_ne(pb, H, tb);
            if (alpha == 0.0 || L1.r == 0 || L2.r == 0) continue;
            Term T;
            T.h = H.m / 2;
            T.row0 = side == 0 ? H.row0 : H.row0 + T.h;
            T.target = side == 0 ? H.nw : H.se;
            T.eps = e2[i];
            const bool left = L1.r < L2.r;            // u copied from L1, v computed
            T.k = left ? L1.r : L2.r;
            double *big, *tmp, *s3;
            if ((rc = ar.alloc(&big, (long long)T.h * T.k)) || (rc = ar.alloc(&tmp, (long long)L1.r * L2.r)) ||
                (rc = ar.alloc(&s3, T.k)))
                return rc;
            T.s = s3;
            if (left) {
                // tmp (r2 x r1) = L2.U^T L1.V ; v3 = alpha L2.V diag(s2) tmp
                g1.push_back({L2.U, L1.V, nullptr, nullptr, tmp, L2.r, L1.r, T.h, T.h, T.h, 0, L2.r, 1, 0, 1.0, 0.0});
                g2.push_back({L2.V, tmp, nullptr, L2.S, big, T.h, L1.r, L2.r, T.h, L2.r, 0, T.h, 0, 0, alpha, 0.0});
                T.u = L1.U;
                T.v = big;
                for (int j = 0; j < T.k; ++j)
                    tnorm.push_back({big + (long long)j * T.h, nullptr, big + (long long)j * T.h, nullptr, s3 + j,
                                     L1.S + j, 1.0, e2[i], 1.0, T.h, kNormU});
            } else {
                // tmp (r1 x r2) = L1.V^T L2.U ; u3 = alpha L1.U diag(s1) tmp
                g1.push_back({L1.V, L2.U, nullptr, nullptr, tmp, L1.r, L2.r, T.h, T.h, T.h, 0, L1.r, 1, 0, 1.0, 0.0});
                g2.push_back({L1.U, tmp, nullptr, L1.S, big, T.h, L2.r, L1.r, T.h, L1.r, 0, T.h, 0, 0, alpha, 0.0});
                T.u = big;
                T.v = L2.V;
                for (int j = 0; j < T.k; ++j)
                    tnorm.push_back({big + (long long)j * T.h, nullptr, big + (long long)j * T.h, nullptr, s3 + j,
                                     L2.S + j, 1.0, e2[i], 1.0, T.h, kNormU});
            }
            term_of[2 * i + side] = (int)terms.size();
            terms.push_back(T);
        }
    }

    // ---- per depth: products of subtrees with low-rank factors
    int levels = 0;
    for (const HDesc &H : nodes) levels = std::max(levels, H.level + 1);
    std::vector<double *> YA(levels, nullptr), YB(levels, nullptr);
    std::vector<int> RA(levels, 0), RB(levels, 0);
    if (alpha != 0.0) {
        for (const HDesc &H : nodes) {
            RA[H.level] = std::max({RA[H.level], op_ne(pb, H, tb).r, op_sw(pb, H, tb).r});
            RB[H.level] = std::max({RB[H.level], op_ne(pa, H, ta).r, op_sw(pa, H, ta).r});
        }
        for (int d = 0; d < levels; ++d) {
            for (int pass = 0; pass < 2; ++pass) {
                const int R = pass == 0 ? RA[d] : RB[d];
                if (R == 0) continue;
                double *X, *Y;
                if ((rc = ar.alloc(&X, (long long)m * R)) || (rc = ar.alloc(&Y, (long long)m * R))) return rc;
                DG_CUDA(cudaMemsetAsync(X, 0, sizeof(double) * (size_t)m * R, st));
                std::vector<CopyJob> cj;
                std::vector<int> cc;
                for (const HDesc &H : nodes) {
                    if (H.level != d) continue;
                    const int h = H.m / 2;
                    // pass 0 (plmm): nw rows <- op(B).ne u-side, se rows <- op(B).sw u-side
                    // pass 1 (lpmm): nw rows <- op(A).sw v-side, se rows <- op(A).ne v-side
                    const View top = pass == 0 ? op_ne(pb, H, tb) : op_sw(pa, H, ta);
                    const View bot = pass == 0 ? op_sw(pb, H, tb) : op_ne(pa, H, ta);
                    const double *st_ = pass == 0 ? top.U : top.V;
                    const double *sb_ = pass == 0 ? bot.U : bot.V;
                    if (top.r) {
                        cj.push_back({st_, X + H.row0, h, m, h});
                        cc.push_back(top.r);
                    }
                    if (bot.r) {
                        cj.push_back({sb_, X + H.row0 + h, h, m, h});
                        cc.push_back(bot.r);
                    }
                }
                if ((rc = launch_copies(ar, cj, cc, st))) return rc;
                // pass 0: op(A) restricted; pass 1: op(B)^T restricted
                const Plan *P = pass == 0 ? pa : pb;
                const int tr = pass == 0 ? ta : !tb;
                if ((rc = restricted_apply(ar, P, tr, d + 1, X, Y, R, alpha, st))) return rc;
                (pass == 0 ? YA : YB)[d] = Y;
            }
        }
    }

    // ---- layout of the result: segments and capacities of every block
    std::vector<DPlrMtx *> lrs, leaves;
    collect(C, lrs, leaves);
    if ((int)lrs.size() != 2 * nH || (int)leaves.size() != nL)
        return fail(DPLR_GPU_EINVAL, "dplrgeppmm: internal structure mismatch");
    const int nb = 2 * nH;
    std::vector<std::vector<Segment>> segs(nb);
    std::vector<int> rank_f(nb, 0);
    for (int i = 0; i < nH; ++i) {
        const HDesc &H = nodes[i];
        for (int side = 0; side < 2; ++side) {
            const int b = side == 0 ? H.ne : H.sw;
            const int old = pc->lr[b].rank;
            std::vector<Segment> &S = segs[b];
            if (beta != 0.0 && old > 0) S.push_back({0, old, -1});
            if (alpha != 0.0) {
                // ne: plmm then lpmm ; sw: lpmm then plmm
                const int rp = (side == 0 ? op_ne(pb, H, tb) : op_sw(pb, H, tb)).r;
                const int rl = (side == 0 ? op_ne(pa, H, ta) : op_sw(pa, H, ta)).r;
                if (side == 0) {
                    if (rp) S.push_back({1, rp, -1});
                    if (rl) S.push_back({2, rl, -1});
                } else {
                    if (rl) S.push_back({2, rl, -1});
                    if (rp) S.push_back({1, rp, -1});
                }
            }
            // ancestor terms, parent first
            int child = i;
            for (int P = H.parent; P >= 0; child = P, P = nodes[P].parent) {
                const int side_p = nodes[P].nw == child ? 0 : 1;
                const int t = term_of[2 * P + side_p];
                if (t >= 0) S.push_back({3, terms[t].k, t});
            }
            for (const Segment &g : S) rank_f[b] += g.count;
        }
    }

    // device result: per block u, v (n x rank), sig; per leaf b x b
    std::vector<long long> off_u(nb), off_v(nb), off_s(nb), off_d(nL);
    long long tot = 0;
    for (int b = 0; b < nb; ++b) {
        const long long n = pc->lr[b].n, r = rank_f[b];
        off_u[b] = tot;
        tot += n * r;
        off_v[b] = tot;
        tot += n * r;
        off_s[b] = tot;
        tot += r;
    }
    for (int l = 0; l < nL; ++l) {
        off_d[l] = tot;
        tot += (long long)pc->leaves[l].b * pc->leaves[l].b;
    }
    double *out;
    if ((rc = ar.alloc(&out, tot))) return rc;

    // ---- 1. leaves: alpha op(A) op(B) + beta C
    std::vector<GemmJob> gl;
    for (int l = 0; l < nL; ++l) {
        const int bl = pc->leaves[l].b;
        if (bl == 0) continue;
        gl.push_back({pa->pool + pa->leaves[l].d, pb->pool + pb->leaves[l].d, pc->pool + pc->leaves[l].d, nullptr,
                      out + off_d[l], bl, bl, bl, bl, bl, bl, bl, ta, tb, alpha, beta});
    }
    if ((rc = launch_gemms(ar, gl, st))) return rc;

    // ---- 3, 4. terms, their normalisation
    if ((rc = launch_gemms(ar, g1, st)) || (rc = launch_gemms(ar, g2, st)) || (rc = launch_cols(ar, tnorm, st)))
        return rc;

    // thresholds of dplrgeprk below a term's target: eps/2 above leaves,
    // eps/4 otherwise, compounded from the target down
    auto f_of = [&](int node) { return nodes[node].nw < 0 ? 2.0 : 4.0; };
    std::vector<ColJob> cols;
    const double bsign = beta < 0.0 ? -1.0 : 1.0, babs = fabs(beta);
    for (int i = 0; i < nH; ++i) {
        const HDesc &H = nodes[i];
        const int h = H.m / 2;
        for (int side = 0; side < 2; ++side) {
            const int b = side == 0 ? H.ne : H.sw;
            const LRDesc &Lc = pc->lr[b];
            int col = 0;
            for (const Segment &g : segs[b]) {
                for (int j = 0; j < g.count; ++j, ++col) {
                    ColJob J{};
                    J.du = out + off_u[b] + (long long)col * h;
                    J.dv = out + off_v[b] + (long long)col * h;
                    J.dsig = out + off_s[b] + col;
                    J.n = h;
                    J.g = 1.0;
                    J.sm = 1.0;
                    if (g.kind == 0) {
                        J.mode = kOld;
                        J.su = pc->pool + Lc.u + (long long)j * h;
                        J.sv = pc->pool + Lc.v + (long long)j * h;
                        J.ss = pc->pool + Lc.sig + j;
                        J.sm = babs;
                        J.g = bsign;
                    } else if (g.kind == 1) {
                        // plmm: u = op(P) L.u (rows of the block's u side), v = L.v
                        const View L = side == 0 ? op_ne(pb, H, tb) : op_sw(pb, H, tb);
                        const int r0 = side == 0 ? H.row0 : H.row0 + h;
                        J.mode = kNormU;
                        J.su = YA[H.level] + r0 + (long long)j * m;
                        J.sv = L.V + (long long)j * h;
                        J.ss = L.S + j;
                        J.thr = e2[i];
                    } else if (g.kind == 2) {
                        // lpmm: u = L.u, v = op(P)^T L.v (rows of the block's v side)
                        const View L = side == 0 ? op_ne(pa, H, ta) : op_sw(pa, H, ta);
                        const int r0 = side == 0 ? H.row0 + h : H.row0;
                        J.mode = kNormV;
                        J.su = L.U + (long long)j * h;
                        J.sv = YB[H.level] + r0 + (long long)j * m;
                        J.ss = L.S + j;
                        J.thr = e2[i];
                    } else {
                        const Term &T = terms[g.term];
                        // u rows: the block's u side, v rows: its v side, relative to the term
                        const int ur = (side == 0 ? H.row0 : H.row0 + h) - T.row0;
                        const int vr = (side == 0 ? H.row0 + h : H.row0) - T.row0;
                        double thr = T.eps;
                        // from the target down to this node
                        std::vector<int> path;
                        for (int q = i;; q = nodes[q].parent) {
                            path.push_back(q);
                            if (q == T.target) break;
                        }
                        for (int q = (int)path.size() - 1; q >= 0; --q) thr /= f_of(path[q]);
                        J.mode = kNormUV;
                        J.su = T.u + ur + (long long)j * T.h;
                        J.sv = T.v + vr + (long long)j * T.h;
                        J.ss = T.s + j;
                        J.thr = thr;
                    }
                    cols.push_back(J);
                }
            }
        }
    }
    if ((rc = launch_cols(ar, cols, st))) return rc;

    // ---- 5. ancestor terms into the leaves, parent first
    std::vector<std::vector<GemmJob>> by_dist;
    for (int l = 0; l < nL; ++l) {
        const LeafDesc &Lf = pc->leaves[l];
        if (Lf.b == 0) continue;
        // the H node whose child this leaf is
        int child = ~l, dist = 0;
        int P = -1;
        for (int i = 0; i < nH; ++i)
            if (nodes[i].nw == ~l || nodes[i].se == ~l) P = i;
        for (; P >= 0; child = P, P = nodes[P].parent) {
            const int side_p = nodes[P].nw == child ? 0 : 1;
            const int t = term_of[2 * P + side_p];
            if (t < 0) continue;
            const Term &T = terms[t];
            const int r = Lf.row0 - T.row0;
            if ((int)by_dist.size() <= dist) by_dist.resize(dist + 1);
            by_dist[dist].push_back({T.u + r, T.v + r, out + off_d[l], T.s, out + off_d[l], Lf.b, Lf.b, T.k, T.h, T.h,
                                     Lf.b, Lf.b, 0, 1, 1.0, 1.0});
            ++dist;
        }
    }
    for (const std::vector<GemmJob> &jobs : by_dist)
        if ((rc = launch_gemms(ar, jobs, st))) return rc;

    // ---- host: DPLR's capacity growth, then the values
    // Grown blocks get fresh buffers (live columns from the device, the rest
    // NaN as dplrresizelr leaves it).  The result comes back in one copy to
    // pinned staging and is spread to the tree's buffers by host threads.
    Staging &sg = staging();
    std::lock_guard<std::mutex> lk(sg.mu);
    if (sg.n < (size_t)tot) {
        if (sg.p) cudaFreeHost(sg.p);
        sg.p = nullptr;
        sg.n = 0;
        const size_t want = std::max<size_t>((size_t)tot, (size_t)tot + (size_t)tot / 2);
        DG_CUDA(cudaMallocHost((void **)&sg.p, sizeof(double) * want));
        sg.n = want;
    }
    DG_CUDA(cudaMemcpyAsync(sg.p, out, sizeof(double) * (size_t)tot, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    struct Piece {
        size_t src;            // offset in the result (doubles); SIZE_MAX: NaN fill
        double *dst;
        size_t count;
    };
    std::vector<Piece> pieces;
    const double qnan = std::nan("");
    const size_t kNaN = (size_t)-1;
    auto add = [&](size_t src, double *dst, size_t count) {
        // at most 256 K doubles per piece, so that threads share big blocks
        for (size_t o = 0; o < count; o += (1u << 18))
            pieces.push_back({src == kNaN ? kNaN : src + o, dst + o, std::min<size_t>(1u << 18, count - o)});
    };
    for (int b = 0; b < nb; ++b) {
        DPlrMtx *L = lrs[b];
        // dplrresizelr at every append that overflows, in DPLR's order
        int cap = L->dlr.capacity, r = 0;
        bool first = true;
        for (const Segment &g : segs[b]) {
            if (first && g.kind == 0) {
                r = g.count;
            } else {
                if (cap < r + g.count) cap = std::max(r + g.count, 2 * cap);
                r += g.count;
            }
            first = false;
        }
        const size_t n = (size_t)L->size, rf = (size_t)rank_f[b];
        if (cap > L->dlr.capacity) {
            double *u = (double *)malloc(sizeof(double) * n * cap);
            double *v = (double *)malloc(sizeof(double) * n * cap);
            double *sg = (double *)malloc(sizeof(double) * cap);
            if (!u || !v || !sg) {
                free(u);
                free(v);
                free(sg);
                return fail(DPLR_GPU_ENOMEM, "dplrgeppmm: host allocation failed");
            }
            free(L->dlr.u);
            free(L->dlr.v);
            free(L->dlr.sig);
            L->dlr.u = u;
            L->dlr.v = v;
            L->dlr.sig = sg;
            L->dlr.capacity = cap;
            add(kNaN, u + n * rf, n * (cap - rf));
            add(kNaN, v + n * rf, n * (cap - rf));
            add(kNaN, sg + rf, cap - rf);
        }
        if (rf) {
            add((size_t)off_u[b], L->dlr.u, n * rf);
            add((size_t)off_v[b], L->dlr.v, n * rf);
            add((size_t)off_s[b], L->dlr.sig, rf);
        }
        L->dlr.rank = (int)rf;
    }
    for (int l = 0; l < nL; ++l) {
        const size_t bl = (size_t)pc->leaves[l].b;
        if (bl) add((size_t)off_d[l], leaves[l]->dd.d, bl * bl);
    }
    const double *stage = sg.p;
    std::atomic<size_t> next{0};
    auto worker = [&]() {
        for (size_t i = next.fetch_add(1); i < pieces.size(); i = next.fetch_add(1)) {
            const Piece &q = pieces[i];
            if (q.src == kNaN) std::fill(q.dst, q.dst + q.count, qnan);
            else memcpy(q.dst, stage + q.src, sizeof(double) * q.count);
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned nt = (unsigned)std::min<size_t>(std::min(16u, hw), std::max<size_t>(1, pieces.size() / 4));
    std::vector<std::thread> th;
    for (unsigned t = 1; t < nt; ++t) th.emplace_back(worker);
    worker();
    for (std::thread &t : th) t.join();
    return 0;
}

const char *variant_name(int ta, int tb)
{
    return ta ? (tb ? "dplrptptmm" : "dplrptpmm") : (tb ? "dplrpptmm" : "dplrppmm");
}

}  // namespace

}  // namespace dg

using namespace dg;

extern "C" {

int dplr_gpu_geppmm(char transa, char transb, int m, double alpha, DPlrMtx *A, DPlrMtx *B, double beta, DPlrMtx *C,
                    double eps, void *stream)
{
    dg::NvtxRange nvtx_("dplr_gpu_geppmm");
    const int ta = transa == 'T' || transa == 't';
    const int tb = transb == 'T' || transb == 't';
    const char *fn = variant_name(ta, tb);
    if (m < 0) return fail(DPLR_GPU_EINVAL, "%s: invalid matrix size %d", fn, m);
    if (!A || !B || !C) return fail(DPLR_GPU_EINVAL, "%s: null argument", fn);
    if (A->type != B->type || B->type != C->type) return fail(DPLR_GPU_EINVAL, "%s: A, B and C type do not match", fn);
    if (A->size != m || B->size != m || C->size != m) return fail(DPLR_GPU_EINVAL, "%s: invalid A, B or C size", fn);
    int rc;
    if ((rc = validate_tree(m, A, fn)) || (rc = validate_tree(m, B, fn)) || (rc = validate_tree(m, C, fn))) return rc;
    if ((rc = same_structure(A, B, C, fn))) return rc;
    if (m == 0) return 0;
    rc = geppmm_device(ta, tb, m, alpha, A, B, beta, C, eps, (cudaStream_t)stream);
    if (rc == 0) recompress_after(m, C);
    return rc;
}

void dplr_gpu_release_staging(void)
{
    Staging &sg = staging();
    std::lock_guard<std::mutex> lk(sg.mu);
    if (sg.p) cudaFreeHost(sg.p);
    sg.p = nullptr;
    sg.n = 0;
}

void dplrgeppmm(char transa, char transb, int m, double *alpha, DPlrMtx *A, DPlrMtx *B, double *beta, DPlrMtx *C,
                double eps)
{
    dg::NvtxRange nvtx_("dplrgeppmm");
    if (dplr_gpu_geppmm(transa, transb, m, *alpha, A, B, *beta, C, eps, nullptr))
        fprintf(stderr, "%s\n", dplr_gpu_last_error());
}

}  // extern "C"
