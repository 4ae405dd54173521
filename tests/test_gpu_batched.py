"""rnla_solve_batched: many independent blendenpik solves, run by a few
workers (host threads with their own streams, grids sized for a share of
the SMs).  Every problem's x must match its own single-problem _dev call to
the solver's accuracy -- same sketch seed and kernels, but the workers'
smaller grids group the per-CTA partial sums differently, so the last bits
can differ -- and LAPACK's residual; a failing problem is reported in its
own status and does not stop the others.  The batch of mixed shapes follows the
batched least-squares workload (m in [1000, 50000], n in [16, 256],
m >= 8 n, kappa 1e6, noise 1e-6), at sizes LAPACK checks in seconds."""
import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _problem(m, n, kappa, noise, seed):
    A = O.make_lowrank_test_matrix(m, n, np.logspace(0, -np.log10(kappa), n), seed + 1, seed + 2)
    rng = np.random.default_rng(seed + 3)
    b = A @ rng.standard_normal(n) + noise * rng.standard_normal(m)
    return A, b


def _relres(A, x, b):
    return np.linalg.norm(A @ np.ravel(x) - b) / np.linalg.norm(b)


def _dev(A, b, f32=False):
    import torch
    a = torch.tensor(np.asfortranarray(A), device="cuda").t().contiguous().t()
    if f32:
        a = a.float()
    return a, torch.tensor(b, device="cuda"), torch.zeros(A.shape[1], dtype=torch.float64, device="cuda")


def _opts(rnla, precision):
    return rnla.options(precision=precision, inner_solver=rnla.InnerSolver.LSQR, atol=1e-14, btol=1e-14)


@pytest.mark.parametrize("precision", ["BF16X", "FP64"])
def test_batch_matches_single_calls(rnla, precision):
    import torch
    prec = getattr(rnla.Precision, precision)
    shapes = [(3000, 40, False), (8000, 100, True), (2400, 256, False), (2000, 17, False)]
    probs, host = [], []
    for i, (m, n, f32) in enumerate(shapes):
        A, b = _problem(m, n, 1e6, 1e-6, seed=10 * i)
        host.append((A, b))
        probs.append(_dev(A, b, f32))
    o = _opts(rnla, prec)
    status, stats = rnla.solve_batched_dev(probs, 1e-12, 2000, 4.0, o)
    torch.cuda.synchronize()
    assert status == [0] * len(shapes)
    for (a, b, x), st, (A, bh) in zip(probs, stats, host):
        x1 = torch.zeros_like(x)
        st1 = rnla.blendenpik_dev(a, b, x1, 1e-12, 2000, 4.0, o)
        torch.cuda.synchronize()
        Ar = a.double().cpu().numpy()
        assert abs(_relres(Ar, x.cpu().numpy(), bh) - _relres(Ar, x1.cpu().numpy(), bh)) < 1e-12
        assert abs(st["iterations"] - st1["iterations"]) <= 2 and st["istop"] == st1["istop"]
    for (A, b), (a, _, x) in zip(host, probs):
        Ar = a.double().cpu().numpy()            # the matrix as stored (f32 rounding included)
        xl = np.linalg.lstsq(Ar, b, rcond=None)[0]
        assert abs(_relres(Ar, x.cpu().numpy(), b) - _relres(Ar, xl, b)) < 1e-10


def test_failing_problems_do_not_stop_the_batch(rnla):
    import torch
    A0, b0 = _problem(1500, 30, 1e4, 1e-6, seed=1)
    As, bs = _problem(900, 12, 1e3, 1e-4, seed=2)
    As[:, 3] = 0.0                                  # exactly singular sketch
    A2, b2 = _problem(2500, 64, 1e5, 1e-6, seed=3)
    probs = [_dev(A0, b0), _dev(A0[:20], b0[:20]), _dev(As, bs), _dev(A2, b2)]
    status, stats = rnla.solve_batched_dev(probs, 1e-12, 2000, 4.0, _opts(rnla, rnla.Precision.BF16X))
    torch.cuda.synchronize()
    assert status == [0, rnla.NotOverdetermined.code, rnla.SingularMatrix.code, 0]
    assert stats[1]["iterations"] == 0
    for (a, b, x), (A, bb) in ((probs[0], (A0, b0)), (probs[3], (A2, b2))):
        xl = np.linalg.lstsq(A, bb, rcond=None)[0]
        assert abs(_relres(A, x.cpu().numpy(), bb) - _relres(A, xl, bb)) < 1e-10


def test_batched_workload_sample(rnla):
    """Twelve problems drawn like the batched workload (shapes resampled
    until m >= 8 n), m capped at 20000 to keep the LAPACK check short."""
    import torch
    rng = np.random.default_rng(12)
    probs, host = [], []
    while len(probs) < 12:
        m, n = int(rng.integers(1000, 20001)), int(rng.integers(16, 257))
        if m < 8 * n:
            continue
        A, b = _problem(m, n, 1e6, 1e-6, seed=100 + len(probs))
        host.append((A, b))
        probs.append(_dev(A, b))
    status, stats = rnla.solve_batched_dev(probs, 1e-12, 2000, 4.0, _opts(rnla, rnla.Precision.BF16X))
    torch.cuda.synchronize()
    assert status == [0] * 12
    for (A, b), (_, _, x), st in zip(host, probs, stats):
        xl = np.linalg.lstsq(A, b, rcond=None)[0]
        assert abs(_relres(A, x.cpu().numpy(), b) - _relres(A, xl, b)) < 1e-10
        assert 0 < st["iterations"] < 200


def test_empty_batch(rnla):
    assert rnla.solve_batched_dev([], 1e-12, 100, 4.0) == ([], [])


def test_cached_memory_release_between_batches(rnla):
    """rnla_release_cached_memory trims the pools; later solves allocate
    again and give the same result."""
    import torch
    A, b = _problem(3000, 50, 1e5, 1e-6, seed=7)
    p1, p2 = _dev(A, b), _dev(A, b)
    o = _opts(rnla, rnla.Precision.BF16X)
    assert rnla.solve_batched_dev([p1], 1e-12, 2000, 4.0, o)[0] == [0]
    torch.cuda.synchronize()
    assert rnla.lib().rnla_release_cached_memory() == 0
    assert rnla.solve_batched_dev([p2], 1e-12, 2000, 4.0, o)[0] == [0]
    torch.cuda.synchronize()
    assert torch.equal(p1[2], p2[2])
