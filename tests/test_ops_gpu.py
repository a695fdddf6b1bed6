"""Device-resident dplr_gpu_scal / dplr_gpu_adpy on plans against the host
drop-ins dplrscal / dplradpy applied to the same tree (apply results agree
to 1e-13), with the factorisation dropped and the float-pair copy following."""
import numpy as np
import pytest
import torch

from dplr_gb300 import gen, tree

pytestmark = pytest.mark.gpu

TREES = {
    "uniform1k": lambda: gen.random_tree(1024, 64, 16, seed=1),
    "uneven2k": lambda: gen.random_tree(2048, 32, [70, 0, 9, 33, 1, 5], seed=2, capacity_extra=3),
    "exp4k": lambda: gen.exp1d_tree(gen.sorted_uniform(4096, 5), 0.1, 1e-2, 64, 8, seed=5),
}


def host_op(t, fn):
    """Apply a host drop-in to a C copy of t and read the tree back."""
    from dplr_gb300 import _native
    a = tree.to_c(t)
    fn(_native.api(), a)
    out = tree.from_c(a)
    tree.free_c(a)
    return out


def applied(plan, x):
    return plan.apply(x).cpu().numpy()


@pytest.mark.parametrize("name", list(TREES))
@pytest.mark.parametrize("alpha", [3.0, -0.5])
def test_device_scal_matches_host(name, alpha):
    from dplr_gb300.plan import GpuPlan
    t = TREES[name]()
    want_tree = host_op(t, lambda api, a: api.scal(t.size, alpha, a))
    x = torch.randn(2, t.size, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(1))
    p, q = GpuPlan(t), GpuPlan(want_tree)
    p.scal(alpha)
    y, want = applied(p, x), applied(q, x)
    assert np.linalg.norm(y - want) <= 1e-13 * np.linalg.norm(want)
    # same factors as the host result, not only the same operator
    assert torch.equal(p.read_pool(), q.read_pool())
    p.close()
    q.close()


@pytest.mark.parametrize("name", list(TREES))
def test_device_adpy_matches_host(name):
    from dplr_gb300.plan import GpuPlan
    t = TREES[name]()
    d = np.random.default_rng(3).standard_normal(t.size)
    want_tree = host_op(t, lambda api, a: api.adpy(t.size, 0.75, d.copy(), a))
    p, q = GpuPlan(t), GpuPlan(want_tree)
    p.adpy(0.75, torch.tensor(d, device="cuda"))
    assert torch.equal(p.read_pool(), q.read_pool())
    p.close()
    q.close()


def test_ops_drop_factorisation_and_refresh_pairs():
    from dplr_gb300 import _native
    from dplr_gb300.plan import GpuPlan
    t = TREES["exp4k"]()
    p = GpuPlan(t)
    p.factor()
    p.prepare_pairs()
    p.scal(-2.0)
    b = torch.randn(1, t.size, dtype=torch.float64, device="cuda")
    out = torch.empty_like(b)
    rc = _native.lib().dplr_gpu_solve(p._h, b"N", 1, b.data_ptr(), t.size, out.data_ptr(), t.size, None)
    assert rc == -6                                  # DPLR_GPU_ESTATE: the factorisation described the old values
    ref = GpuPlan(t)
    y_ref = -2.0 * ref.apply(b)
    y = p.apply(b)                                   # the pair copy follows the scaled values
    assert float((y - y_ref).norm() / y_ref.norm()) <= 1e-13
    p.factor()                                       # and a new factorisation solves the scaled matrix
    x = p.solve(b)
    assert float((p.apply(x) - b).norm() / b.norm()) <= 1e-10
    p.close()
    ref.close()
