// factor.cuh -- Woodbury factorisation state shared by factor.cu,
// solve.cu and inverse.cu.
#pragma once

#include "internal.cuh"

namespace dg {

struct LevelOps {
    Schedule n;       // op N: panels on V, caps K^-1, updates with Z_l
    Schedule t;       // op T: panels on Z_l, caps S K^-T, updates with V
    int width = 0;    // r_l
    std::vector<int> blocks;   // LRDesc indices at this level
    std::vector<int> nodes;    // HDesc indices at this level
};

struct ScatterItem;

struct Fact {
    int flags = 0;
    bool transposed = false;
    // the numbers are current (cleared when the plan's values change; the
    // layout below is kept and reused by the next factorisation)
    bool valid = false;
    int key_chunk = 0, key_nb = 0;    // schedule parameters the layout was built with
    // per level: the level right-hand side's scatter items (U: [0], V: [1])
    // and the capacitance inverses (offsets, orders, node ids), all levels
    // in one device array each
    ScatterItem *d_scat = nullptr;
    std::vector<int> scat_begin[2], scat_count[2], scat_max[2];
    long long *d_inv_off = nullptr;
    int *d_inv_size = nullptr;
    std::vector<int> inv_begin, inv_count, inv_max, inv_ids;
    std::vector<LevelOps> lv;
    std::vector<long long> zoff;      // per level, offset in zpool / ztpool
    long long zdoubles = 0;
    double *zpool = nullptr, *ztpool = nullptr;
    std::vector<long long> koff;      // per node
    long long kdoubles = 0;
    double *kpool = nullptr;
    std::vector<long long> leafoff;
    long long leafdoubles = 0;
    double *leafinv = nullptr;
    Schedule leafN, leafT;            // expand schedules of the leaf step
    // batched inverse tables
    long long *d_koff = nullptr, *d_leafoff = nullptr;
    int *d_ksize = nullptr, *d_leafsize = nullptr, *d_info = nullptr;
    // scratch
    double *work = nullptr;
    size_t work_doubles = 0;
    double *rhs = nullptr;            // factorisation right-hand sides (m x r_max)
    size_t rhs_doubles = 0;
    double *vec = nullptr;            // refinement vectors
    size_t vec_doubles = 0;
    double *gtr = nullptr;            // the transposed sweep's running right-hand side
    size_t gtr_doubles = 0;
    long long bytes = 0;
    // first singular matrix met while factoring: 0 none, 1 leaf, 2 capacitance
    int sing_kind = 0, sing_index = -1, sing_info = 0;
};


int factor_build(Plan *p, int flags, cudaStream_t st);
void factor_free(Plan *p);
// The plan's values changed: the factorisation's numbers are stale; its
// layout is kept for the next factor_build.
void factor_invalidate(Plan *p);
// The plan's factorisation when its numbers are current, else nullptr.
Fact *factor_of(const Plan *p);
int factor_solve(Plan *p, int trans, int nrhs, const double *B, int ldb, double *X, int ldx,
                 cudaStream_t st);
long long factor_bytes(const Plan *p);
int axpby_device(int m, int n, double a, const double *X, int ldx, double b, double *Y, int ldy,
                 cudaStream_t st);
int refine_fixed(Plan *p, int n, const double *B, int ldb, double *X, int ldx, int corrections, cudaStream_t st);

}  // namespace dg
