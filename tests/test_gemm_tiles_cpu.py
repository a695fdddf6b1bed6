"""Host logic of the batched FP64 GEMM (dplr_gb300/csrc/gemm.cuh): the tile
and split-K planner must cover every output element and every k of every
job exactly once, with disjoint partial-sum regions for split jobs.  A
host-only program including the header is built with nvcc and run on the
CPU (no kernel is launched)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "dplr_gb300", "csrc")

PROGRAM = r'''
#include "gemm.cuh"
#include <cstdio>
#include <random>
using namespace dg;
int main() {
    std::mt19937 rng(7);
    std::vector<GemmJob> jobs;
    int shapes[][3] = {{1, 1, 1}, {64, 64, 16}, {65, 63, 17}, {256, 256, 256}, {64, 64, 8192},
                       {17, 33, 4097}, {128, 128, 1024}, {512, 40, 3000}, {3, 5, 0}, {200, 1, 70000}};
    for (auto &s : shapes) {
        GemmJob J{};
        J.M = s[0]; J.N = s[1]; J.K = s[2];
        jobs.push_back(J);
    }
    for (int r = 0; r < 40; ++r) {
        GemmJob J{};
        J.M = 1 + rng() % 300; J.N = 1 + rng() % 300; J.K = rng() % 20000;
        jobs.push_back(J);
    }
    std::vector<GemmTile> tiles;
    std::vector<GemmRed> reds;
    long long ptot = 0;
    plan_gemm_tiles(jobs, tiles, reds, ptot);
    // per job: count coverage of (i, j) x k-range, partial regions
    for (int j = 0; j < (int)jobs.size(); ++j) {
        const GemmJob &J = jobs[j];
        std::vector<int> kcov((size_t)J.K + 1, 0);
        long long cells = 0;
        int split = 0;
        for (const GemmTile &t : tiles) {
            if (t.job != j) continue;
            if (t.i0 % kGT || t.j0 % kGT || t.i0 >= J.M || t.j0 >= J.N) { printf("bad tile origin\n"); return 1; }
            if (t.k0 < 0 || t.k1 > J.K || t.k0 > t.k1 || (t.k0 % kGK)) { printf("bad k range\n"); return 1; }
            if (t.i0 == 0 && t.j0 == 0) for (int k = t.k0; k < t.k1; ++k) kcov[k]++;
            cells += (long long)std::min(kGT, J.M - t.i0) * std::min(kGT, J.N - t.j0);
            if (t.p >= 0) split = 1;
        }
        for (int k = 0; k < J.K; ++k) if (kcov[k] != 1) { printf("job %d k %d covered %d\n", j, k, kcov[k]); return 1; }
        // tiles per k-slice times cells: every (i, j) once per slice
        int slices = 0;
        for (const GemmTile &t : tiles) if (t.job == j && t.i0 == 0 && t.j0 == 0) ++slices;
        if (cells != (long long)slices * J.M * J.N) { printf("job %d cells %lld\n", j, cells); return 1; }
        int nred = 0;
        for (const GemmRed &r : reds) if (r.job == j) { ++nred; if (r.slices != slices) { printf("slices\n"); return 1; } }
        if (split != (nred == 1) || (slices > 1) != split) { printf("job %d split bookkeeping\n", j); return 1; }
    }
    // partial regions of split jobs are disjoint and inside ptot
    long long end = 0;
    for (const GemmRed &r : reds) {
        const GemmJob &J = jobs[r.job];
        if (r.p < end) { printf("overlap\n"); return 1; }
        end = r.p + (long long)r.slices * J.M * J.N;
    }
    if (end != ptot) { printf("ptot %lld end %lld\n", ptot, end); return 1; }
    printf("ok %zu tiles %zu splits\n", tiles.size(), reds.size());
    return 0;
}
'''


def test_tiles_cover_every_element_and_k_once(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    src = tmp_path / "tiles.cu"
    src.write_text(PROGRAM)
    exe = tmp_path / "tiles"
    build = subprocess.run([nvcc, "-std=c++17", "-O1", "-gencode", "arch=compute_103a,code=sm_103a",
                            f"-I{CSRC}", str(src), "-o", str(exe)], capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert run.returncode == 0 and run.stdout.startswith("ok"), run.stdout + run.stderr
