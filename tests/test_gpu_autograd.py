"""GPU checks of the differentiable jagged operations (awkward_gb300.autograd).

References:
* a padded dense torch implementation of each op (lists as rows of an
  [nlists, max_len] tensor with masking), differentiated by torch autograd;
* float64 central finite differences (h = 1e-6) of the library's own
  float64 forward kernels along random directions, on a 10,000-list subset
  (directional derivatives <grad f, v> of f = sum(w * op(x)));
* at the full differentiable-ops size (4,000,000 lists, Poisson(16) lengths,
  float32), the backward that recomputes the softmax maxima and
  normalisers (forced by the 256 MB activation budget) against the one that
  keeps y.

Tolerances: float64 1e-12 relative against the dense reference, float32
1e-5 relative (softmax 2e-6 absolute on probabilities); finite differences
within 1e-6 relative of the analytic directional derivative.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _jagged(nl, lam, seed, dtype, base=0, extra=None):
    import torch

    rng = np.random.default_rng(seed)
    L = rng.poisson(lam, nl)
    L[rng.random(nl) < 0.02] = 0
    if extra is not None:
        L = np.concatenate([L, extra])
    off = (np.concatenate([[0], np.cumsum(L)]) + base).astype(np.int64)
    x = rng.standard_normal(int(off[-1])).astype(dtype)
    return torch.from_numpy(x).cuda(), torch.from_numpy(off).cuda(), L


def _dense(values, offsets):
    """(dense [n, m] view builder, mask) for a jagged array (offsets may start > 0)."""
    import torch

    L = offsets[1:] - offsets[:-1]
    n = L.numel()
    m = int(L.max().item()) if n else 0
    owner = torch.repeat_interleave(torch.arange(n, device=values.device), L)
    pos = torch.arange(owner.numel(), device=values.device) - (offsets[:-1] - offsets[0])[owner]
    mask = torch.zeros(n, max(m, 1), dtype=torch.bool, device=values.device)
    mask[owner, pos] = True

    def build(v, fill):
        d = torch.full((n, max(m, 1)), fill, dtype=v.dtype, device=v.device)
        return d.index_put((owner, pos), v[int(offsets[0]):int(offsets[-1])])

    return build, mask


def _ref(op, values, offsets):
    import torch

    build, mask = _dense(values, offsets)
    if op == "sum":
        return build(values, 0.0).sum(1)
    if op == "max":
        return build(values, -float("inf")).max(1).values
    d = build(values, -float("inf"))
    y = torch.softmax(d, 1)
    y = torch.where(mask, y, torch.zeros_like(y))
    full = torch.zeros_like(values)
    return full.index_put((torch.arange(int(offsets[0]), int(offsets[-1]), device=values.device),),
                          y[mask])


def _ours(op, values, offsets):
    from awkward_gb300 import autograd as ag

    if op == "sum":
        return ag.segment_sum(values, offsets)
    if op == "max":
        return ag.segment_max(values, offsets)
    return ag.jagged_softmax(values, offsets)


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
@pytest.mark.parametrize("op", ["sum", "max", "softmax"])
def test_forward_backward_match_dense_reference(op, dtype):
    import torch

    x, off, _L = _jagged(10_000, 16, 1, dtype, base=3, extra=np.array([0, 1, 300, 0, 2]))
    xg = x.clone().requires_grad_(True)
    y = _ours(op, xg, off)
    g = torch.randn(y.shape, dtype=y.dtype, device="cuda")
    (y * g).sum().backward()
    xr = x.clone().requires_grad_(True)
    yr = _ref(op, xr, off)
    (yr * g).sum().backward()
    tol = dict(rtol=1e-12, atol=1e-12) if dtype == np.float64 else dict(rtol=1e-5, atol=2e-6)
    if op == "max":
        nonempty = (off[1:] - off[:-1]) > 0
        torch.testing.assert_close(y[nonempty], yr[nonempty], rtol=0, atol=0)
        assert bool(torch.isinf(y[~nonempty]).all())
    else:
        torch.testing.assert_close(y, yr, **tol)
    torch.testing.assert_close(xg.grad, xr.grad, **tol)


@pytest.mark.parametrize("op", ["sum", "max", "softmax"])
def test_one_long_list(op):
    import torch

    x, off, _L = _jagged(0, 16, 3, np.float32, extra=np.array([100_000]))
    xg = x.clone().requires_grad_(True)
    y = _ours(op, xg, off)
    g = torch.randn(y.shape, dtype=y.dtype, device="cuda")
    (y * g).sum().backward()
    xr = x.double().clone().requires_grad_(True)
    yr = {"sum": lambda t: t.sum().reshape(1), "max": lambda t: t.max().reshape(1),
          "softmax": lambda t: torch.softmax(t, 0)}[op](xr)
    (yr * g.double()).sum().backward()
    # float32 accumulation over 100,000 elements: sum within 1e-3 relative / 1e-2 absolute
    ytol = {"sum": dict(rtol=1e-3, atol=1e-2), "max": dict(rtol=0, atol=0),
            "softmax": dict(rtol=1e-4, atol=1e-9)}[op]
    gtol = {"sum": dict(rtol=0, atol=0), "max": dict(rtol=0, atol=0),
            "softmax": dict(rtol=1e-4, atol=1e-8)}[op]
    torch.testing.assert_close(y.double(), yr, **ytol)
    torch.testing.assert_close(xg.grad.double(), xr.grad, **gtol)


@pytest.mark.parametrize("op", ["sum", "max", "softmax"])
def test_directional_finite_differences_float64(op):
    import torch

    x, off, _L = _jagged(10_000, 16, 2, np.float64)
    w = None
    h = 1e-6
    for trial in range(3):
        gen = torch.Generator(device="cuda").manual_seed(100 + trial)
        v = torch.randn(x.shape, dtype=torch.float64, device="cuda", generator=gen)
        xg = x.clone().requires_grad_(True)
        y = _ours(op, xg, off)
        if w is None:
            w = torch.randn(y.shape, dtype=torch.float64, device="cuda", generator=gen)
        # empty lists have max -inf: they are left out of f (constant, no gradient)
        fin = torch.isfinite(y.detach())
        (torch.where(fin, y, torch.zeros_like(y)) * w).sum().backward()
        analytic = float((xg.grad * v).sum())
        with torch.no_grad():
            fp = float((_ours(op, x + h * v, off)[fin] * w[fin]).sum())
            fm = float((_ours(op, x - h * v, off)[fin] * w[fin]).sum())
        fd = (fp - fm) / (2 * h)
        assert abs(fd - analytic) <= 1e-6 * max(1.0, abs(analytic)), (op, fd, analytic)


def test_full_size_softmax_recompute_matches_saved():
    import torch

    from awkward_gb300 import autograd as ag

    x, off, _L = _jagged(4_000_000, 16, 5, np.float32)
    g = torch.randn(x.shape, dtype=torch.float32, device="cuda")
    outs = []
    for budget in (ag.DEFAULT_ACTIVATION_BUDGET, 2**40):
        xg = x.clone().requires_grad_(True)
        y = ag.jagged_softmax(xg, off, budget)
        (y * g).sum().backward()
        outs.append((y.detach(), xg.grad))
    # the default budget (256 MB) cannot hold y + statistics at this size
    assert (x.numel() + 2 * (off.numel() - 1)) * 4 > ag.DEFAULT_ACTIVATION_BUDGET
    torch.testing.assert_close(outs[0][0], outs[1][0], rtol=0, atol=0)
    torch.testing.assert_close(outs[0][1], outs[1][1], rtol=1e-5, atol=1e-6)
    # softmax rows sum to one
    sums = torch.zeros(off.numel() - 1, dtype=torch.float64, device="cuda")
    owner = torch.repeat_interleave(torch.arange(off.numel() - 1, device="cuda"), off[1:] - off[:-1])
    sums.index_add_(0, owner, outs[0][0].double())
    nonempty = (off[1:] - off[:-1]) > 0
    torch.testing.assert_close(sums[nonempty], torch.ones_like(sums[nonempty]), rtol=0, atol=1e-5)


def test_full_size_sum_and_max_backward():
    import torch

    from awkward_gb300 import autograd as ag

    x, off, _L = _jagged(4_000_000, 16, 6, np.float32)
    owner = torch.repeat_interleave(torch.arange(off.numel() - 1, device="cuda"), off[1:] - off[:-1])
    xg = x.clone().requires_grad_(True)
    s = ag.segment_sum(xg, off)
    g = torch.randn(s.shape, dtype=torch.float32, device="cuda")
    (s * g).sum().backward()
    assert torch.equal(xg.grad, g[owner])
    xg2 = x.clone().requires_grad_(True)
    m = ag.segment_max(xg2, off)
    (m * g).sum().backward()
    nonempty = (off[1:] - off[:-1]) > 0
    # exactly one element per non-empty list receives its list's gradient: the first maximum
    nz = xg2.grad != 0
    assert int(nz.sum()) <= int(nonempty.sum())
    assert torch.equal(x[nz], m[owner[nz]])
    torch.testing.assert_close(xg2.grad.sum().double(), g[nonempty].sum().double(), rtol=1e-5, atol=1e-3)


@pytest.mark.parametrize("op", ["sum", "softmax"])
def test_elements_outside_the_lists_get_zero_gradients(op):
    """Outputs are allocated uninitialised; the kernels must set the elements
    no list covers (before offsets[0] and after offsets[-1]) to 0."""
    import torch

    from awkward_gb300 import autograd as ag

    n_vals = 50_000
    garbage = torch.full((4 * n_vals,), float("nan"), device="cuda")
    del garbage  # its memory goes back to the caching allocator, still NaN
    L = torch.full((4000,), 10, dtype=torch.int64, device="cuda")
    off = torch.zeros(4001, dtype=torch.int64, device="cuda")
    torch.cumsum(L, 0, out=off[1:])
    off += 123  # 123 leading and n_vals - 40123 trailing uncovered elements
    x = torch.randn(n_vals, dtype=torch.float32, device="cuda").requires_grad_(True)
    y = ag.segment_sum(x, off) if op == "sum" else ag.jagged_softmax(x, off)
    y.backward(torch.ones_like(y))
    inside = torch.zeros(n_vals, dtype=torch.bool, device="cuda")
    inside[123:40123] = True
    assert bool((x.grad[~inside] == 0).all())
    assert bool(torch.isfinite(x.grad[inside]).all())
    if op == "softmax":
        assert bool((y[~inside] == 0).all())
