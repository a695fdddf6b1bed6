"""The batched SVD kernel's algorithm (dplr_gb300/csrc/svdbatch.cuh), checked
on the CPU through a numpy mirror of its steps: the round-robin pair
schedule, the two negligibility rules, the sweep bound and the truncated
SVD it produces.  The GPU kernel itself is held to the recompression and
compression restatements in test_recompress.py and test_compress.py.
"""
import os
import re

import numpy as np
import pytest

from dplr_gb300 import gen

HDR = os.path.join(os.path.dirname(__file__), "..", "dplr_gb300", "csrc", "svdbatch.cuh")
U_ROUND = 1.1102230246251565e-16


def _constant(name):
    text = open(HDR).read()
    m = re.search(r"constexpr int %s = (\d+);" % name, text)
    assert m, name
    return int(m.group(1))


MAX_RANK = _constant("kSvdBatchRank")
MAX_SWEEPS = _constant("kSvdSweeps")


def _pair(pi, k, rp):
    m = rp - 1
    if pi == 0:
        return k, m
    return (k + pi) % m, (k - pi + m) % m


def _house_qr(a):
    """In place, the kernel's convention; columns below 2^-60 ||A||_F take no
    reflector."""
    n, r = a.shape
    tau = np.zeros(r)
    negligible = 2.0 ** -60 * np.sqrt(np.sum(a * a))
    for j in range(r):
        x = a[j + 1:, j]
        amax = np.max(np.abs(x)) if x.size else 0.0
        ss = np.sum((x / amax) ** 2) if amax > 0 else 0.0
        alpha = a[j, j]
        nrm = np.hypot(alpha, amax * np.sqrt(ss))
        if amax > 0 and nrm > negligible:
            beta = -np.copysign(nrm, alpha)
            tau[j] = (beta - alpha) / beta
            a[j + 1:, j] *= 1.0 / (alpha - beta)
            a[j, j] = beta
            v = np.concatenate([[1.0], a[j + 1:, j]])
            w = tau[j] * (v @ a[j:, j + 1:])
            a[j:, j + 1:] -= np.outer(v, w)
    return tau


def _house_apply(a, tau, y):
    r = a.shape[1]
    for j in range(r - 1, -1, -1):
        if tau[j] != 0:
            v = np.concatenate([[1.0], a[j + 1:, j]])
            y[j:] -= np.outer(v, tau[j] * (v @ y[j:]))


def _svd_batch(u, sig, v, eps):
    """(U', sig', V', sweeps) as svd_batch_kernel computes them."""
    n, r = u.shape
    a, b = u * sig, v.copy()
    tu, tv = _house_qr(a), _house_qr(b)
    c = np.triu(a[:r, :r]) @ np.triu(b[:r, :r]).T
    jm = np.eye(r)
    tol = 4.0 * r * U_ROUND
    z2 = (r * U_ROUND) ** 2 * np.sum(c * c)
    rp = r + (r & 1)
    for sweep in range(1, MAX_SWEEPS + 1):
        rotated = False
        for k in range(rp - 1):
            for pi in range(rp // 2):
                p, q = _pair(pi, k, rp)
                if p >= r or q >= r:
                    continue
                al, be, ga = c[:, p] @ c[:, p], c[:, q] @ c[:, q], c[:, p] @ c[:, q]
                if al <= z2 or be <= z2 or not abs(ga) > tol * np.sqrt(al) * np.sqrt(be):
                    continue
                zeta = (be - al) / (2.0 * ga)
                t = 0.5 / zeta if abs(zeta) > 1e150 else np.copysign(1.0, zeta) / (abs(zeta) + np.sqrt(1 + zeta * zeta))
                cs = 1.0 / np.sqrt(1.0 + t * t)
                sn = cs * t
                for m in (c, jm):
                    x, y = m[:, p].copy(), m[:, q].copy()
                    m[:, p], m[:, q] = cs * x - sn * y, sn * x + cs * y
                rotated = True
        if not rotated:
            break
    else:
        raise AssertionError("not converged")
    sv = np.sqrt(np.sum(c * c, axis=0))
    order = sorted(range(r), key=lambda i: (-sv[i], i))
    rank = 0
    while rank < r and not sv[order[rank]] < eps:
        rank += 1
    keep = order[:rank]
    inv = np.array([1.0 / sv[i] if sv[i] > 0 else 0.0 for i in keep])
    yu = np.zeros((n, rank))
    yu[:r] = c[:, keep] * inv
    _house_apply(a, tu, yu)
    yv = np.zeros((n, rank))
    yv[:r] = jm[:, keep]
    _house_apply(b, tv, yv)
    return yu, sv[keep], yv, sweep


@pytest.mark.parametrize("rp", list(range(2, MAX_RANK + 2, 2)))
def test_round_robin_meets_every_pair_once(rp):
    seen = set()
    for k in range(rp - 1):
        cols = []
        for pi in range(rp // 2):
            p, q = _pair(pi, k, rp)
            assert p != q
            cols += [p, q]
            seen.add((min(p, q), max(p, q)))
        assert sorted(cols) == list(range(rp))          # disjoint pairs in a round
    assert len(seen) == rp * (rp - 1) // 2


def _cases():
    rng = np.random.default_rng(21)
    # random factors, sig over 12 decades
    u, v = rng.standard_normal((300, 64)), rng.standard_normal((300, 64))
    yield "random64", u, 10.0 ** -rng.uniform(0, 12, 64), v, 1e-10
    # appended copies (what an axpy without recompression leaves)
    u, v = rng.standard_normal((200, 11)), rng.standard_normal((200, 11))
    s = np.abs(rng.standard_normal(11)) * 10.0 ** -rng.uniform(0, 6, 11)
    yield "repeated", np.hstack([u] * 6)[:, :64], np.concatenate([s] * 6)[:64], np.hstack([v] * 6)[:, :64], 1e-9
    # geometric decay with orthonormal factors
    u = np.linalg.qr(rng.standard_normal((128, 40)))[0]
    v = np.linalg.qr(rng.standard_normal((128, 40)))[0]
    yield "decay", u, 0.5 ** np.arange(40), v, 1e-8
    # a dense kernel block given as A I^T (the compression's use)
    x = gen.sorted_uniform(128, seed=11)
    a = gen.exp_kernel_1d(x, 0.1, 1e-2)[:64, 64:].copy()
    yield "dense", a, np.ones(64), np.eye(64), 1e-10


@pytest.mark.parametrize("name,u,s,v,eps", list(_cases()), ids=[c[0] for c in _cases()])
def test_mirror_is_the_truncated_svd_within_the_sweep_bound(name, u, s, v, eps):
    m = (u * s) @ v.T
    uo, so, vo, sweeps = _svd_batch(u.copy(), s.copy(), v.copy(), eps)
    assert sweeps <= MAX_SWEEPS // 2, sweeps
    uf, sf, vtf = np.linalg.svd(m)
    k = int(np.sum(sf >= eps))
    assert len(so) == k
    scale = max(1.0, sf[0])
    np.testing.assert_allclose(so, sf[:k], rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose((uo * so) @ vo.T, (uf[:, :k] * sf[:k]) @ vtf[:k], rtol=0, atol=1e-13 * scale)
    np.testing.assert_allclose(uo.T @ uo, np.eye(k), atol=1e-12)
    np.testing.assert_allclose(vo.T @ vo, np.eye(k), atol=1e-12)


def test_mirror_keeps_zero_blocks_at_rank_zero():
    rng = np.random.default_rng(3)
    uo, so, vo, _ = _svd_batch(rng.standard_normal((32, 5)), np.zeros(5), rng.standard_normal((32, 5)), 1e-12)
    assert len(so) == 0
