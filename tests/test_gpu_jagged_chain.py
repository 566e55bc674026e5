"""GPU parity of the jagged slicing chain (array[mask], array[idx], array[..., 1:]).

* ``jagged_mask_to_index`` against numpy (positions of true entries within
  their lists, offsets = cumulative counts), bit-exact, including empty lists,
  offsets not starting at 0, an all-true / all-false mask and a 100,000-element
  list;
* ``take`` against numpy for 1, 2, 4 and 8-byte items, and its range error;
* the whole chains at moderate size against the C oracle's
  ``jagged_apply`` / ``next_range`` and numpy gathers, bit-exact;
* at the full jagged-slicing size (10,000,000 lists, Poisson(8), float32
  content), exact properties: the mask chain's carry equals the positions of
  the true entries, the index chain's carry equals start + (idx mod len), and
  the [..., 1:] chain keeps every inner element but the first.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


def _case(nl, seed, lam=8, base=0, extra=None, p=0.4, pe=0.01):
    rng = np.random.default_rng(seed)
    L = rng.poisson(lam, nl)
    L[rng.random(nl) < pe] = 0
    if extra is not None:
        L = np.concatenate([L, extra])
    off = (np.concatenate([[0], np.cumsum(L)]) + base).astype(np.int64)
    x = (rng.exponential(1.0, int(off[-1])) * 20).astype(np.float32)
    mask = rng.random(int(off[-1])) < p
    return rng, L, off, x, mask


def _np_mask_index(off, mask):
    L = np.diff(off)
    cs = np.concatenate([[0], np.cumsum(mask[off[0]:].astype(np.int64))])
    counts = cs[off[1:] - off[0]] - cs[off[:-1] - off[0]]
    ioff = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    owner = np.repeat(np.arange(len(L)), L)
    local = np.arange(int(off[-1] - off[0])) - (off[:-1] - off[0])[owner]
    return ioff, local[mask[off[0]:]].astype(np.int64)


@pytest.mark.parametrize("variant", ["poisson", "base", "all_true", "all_false", "long_list",
                                     "short", "half_empty", "tile_cap"])
def test_mask_to_index_matches_numpy(variant):
    import torch

    from awkward_gb300 import jagged

    kw = {"poisson": {}, "base": {"base": 7}, "all_true": {"p": 1.1}, "all_false": {"p": -1},
          "long_list": {"extra": np.array([0, 100_000, 3])},
          # more than 31 lists ending in one 32-element step; runs of empty lists
          "short": {"lam": 0.4}, "half_empty": {"pe": 0.5},
          # tiles of 1024 lists on both sides of the 16384-element staging limit
          "tile_cap": {"lam": 16}}[variant]
    _rng, _L, off, _x, mask = _case(50_000, 11, **kw)
    ioff, idx = jagged.jagged_mask_to_index(torch.from_numpy(off).cuda(),
                                            torch.from_numpy(mask).cuda())
    e_ioff, e_idx = _np_mask_index(off, mask)
    np.testing.assert_array_equal(ioff.cpu().numpy(), e_ioff)
    np.testing.assert_array_equal(idx.cpu().numpy(), e_idx)


@pytest.mark.parametrize("dt", [np.int8, np.int16, np.float32, np.float64])
def test_take_matches_numpy(dt):
    import torch

    from awkward_gb300 import jagged

    rng = np.random.default_rng(5)
    content = rng.integers(-100, 100, 100_003).astype(dt)
    carry = rng.integers(0, len(content), 777_777).astype(np.int64)
    got = jagged.take(torch.from_numpy(content).cuda(), torch.from_numpy(carry).cuda())
    np.testing.assert_array_equal(got.cpu().numpy(), content[carry])
    with pytest.raises(ValueError, match="index out of range"):
        jagged.take(torch.from_numpy(content).cuda(),
                    torch.tensor([0, len(content)], dtype=torch.int64, device="cuda"))


def _oracle_apply(off, ioff, idx):
    n = len(off) - 1
    too = np.zeros(n + 1, np.int64)
    toc = np.zeros(max(len(idx), 1), np.int64)
    msg = oracle.call(oracle.load(), "awkward_ListArray64_getitem_jagged_apply_64", tooffsets=too,
                      tocarry=toc, slicestarts=ioff[:-1].copy(), slicestops=ioff[1:].copy(),
                      sliceouterlen=n, sliceindex=idx, sliceinnerlen=len(idx),
                      fromstarts=off[:-1].copy(), fromstops=off[1:].copy(),
                      contentlen=int(off[-1]))[0]
    assert msg is None
    return too, toc[: len(idx)]


def test_mask_chain_matches_oracle():
    import torch

    from awkward_gb300 import jagged

    _rng, _L, off, x, mask = _case(200_000, 12, base=3)
    too, content = jagged.getitem_jagged_mask(torch.from_numpy(off).cuda(),
                                              torch.from_numpy(x).cuda(),
                                              torch.from_numpy(mask).cuda())
    ioff, idx = _np_mask_index(off, mask)
    e_too, e_carry = _oracle_apply(off, ioff, idx)
    np.testing.assert_array_equal(too.cpu().numpy(), e_too)
    np.testing.assert_array_equal(content.cpu().numpy(), x[e_carry])


def _index_case(rng, L):
    K = np.where(L > 0, rng.poisson(2, len(L)), 0)
    ioff = np.concatenate([[0], np.cumsum(K)]).astype(np.int64)
    idx = np.concatenate([rng.integers(-l, l, k) for l, k in zip(L, K) if k] or
                         [np.zeros(0, np.int64)]).astype(np.int64)
    return ioff, idx


def test_index_chain_matches_oracle():
    import torch

    from awkward_gb300 import jagged

    rng, L, off, x, _mask = _case(200_000, 13)
    ioff, idx = _index_case(rng, L)
    too, content = jagged.getitem_jagged_index(torch.from_numpy(off).cuda(),
                                               torch.from_numpy(x).cuda(),
                                               torch.from_numpy(ioff).cuda(),
                                               torch.from_numpy(idx).cuda())
    e_too, e_carry = _oracle_apply(off, ioff, idx)
    np.testing.assert_array_equal(too.cpu().numpy(), e_too)
    np.testing.assert_array_equal(content.cpu().numpy(), x[e_carry])


@pytest.mark.parametrize("pattern", ["sparse_long", "mixed"])
def test_apply_and_range_slot_search_branches(pattern):
    """Tiles of 1024 lists with at least 1.5 output slots per list fill their
    outputs in warp steps of 32 slots: the lanes' lists come from a popcount of
    the list ends inside the step, a shuffle search when empty lists share an
    end, and a per-lane walk when 32 or more lists end inside one step.  A long
    list followed by 63 empty ones puts 32+ ends in one step; the mixed pattern
    interleaves all three cases."""
    import torch

    from awkward_gb300 import jagged

    rng = np.random.default_rng(16)
    if pattern == "sparse_long":
        L = np.zeros(64 * 2000, np.int64)
        L[::64] = rng.integers(100, 300, 2000)
    else:
        L = rng.poisson(3, 200_000)
        L[rng.random(len(L)) < 0.3] = 0
        runs = rng.integers(0, len(L) - 80, 400)
        for r0 in runs:
            L[r0:r0 + 40 + int(rng.integers(0, 40))] = 0
            L[r0] = int(rng.integers(50, 400))
    off = np.concatenate([[0], np.cumsum(L)]).astype(np.int64)
    x = rng.standard_normal(int(off[-1])).astype(np.float32)
    # every position of every list, as a jagged index: slots = elements
    ioff = off.copy()
    idx = np.concatenate([np.arange(l) for l in L if l] or [np.zeros(0, np.int64)]).astype(np.int64)
    too, content = jagged.getitem_jagged_index(torch.from_numpy(off).cuda(),
                                               torch.from_numpy(x).cuda(),
                                               torch.from_numpy(ioff).cuda(),
                                               torch.from_numpy(idx).cuda())
    e_too, e_carry = _oracle_apply(off, ioff, idx)
    np.testing.assert_array_equal(too.cpu().numpy(), e_too)
    np.testing.assert_array_equal(content.cpu().numpy(), x[e_carry])
    # [..., 1:] on the same lists
    nxo, nxc = jagged.inner_range(torch.from_numpy(off).cuda(), 1, None, None)
    n = len(off) - 1
    lib = oracle.load()
    cl = np.zeros(1, np.int64)
    assert oracle.call(lib, "awkward_ListArray64_getitem_next_range_carrylength", carrylength=cl,
                       fromstarts=off[:-1].copy(), fromstops=off[1:].copy(), lenstarts=n,
                       start=1, stop=jagged.SLICE_NONE, step=1)[0] is None
    e_off = np.zeros(n + 1, np.int64)
    e_carry2 = np.zeros(max(int(cl[0]), 1), np.int64)
    assert oracle.call(lib, "awkward_ListArray64_getitem_next_range_64", tooffsets=e_off,
                       tocarry=e_carry2, fromstarts=off[:-1].copy(), fromstops=off[1:].copy(),
                       lenstarts=n, start=1, stop=jagged.SLICE_NONE, step=1)[0] is None
    np.testing.assert_array_equal(nxo.cpu().numpy(), e_off)
    np.testing.assert_array_equal(nxc.cpu().numpy(), e_carry2[: int(cl[0])])


def test_index_chain_error_is_awkwards():
    import torch

    from awkward_gb300 import jagged

    off = torch.tensor([0, 2, 5], dtype=torch.int64, device="cuda")
    x = torch.zeros(5, dtype=torch.float32, device="cuda")
    ioff = torch.tensor([0, 1, 2], dtype=torch.int64, device="cuda")
    idx = torch.tensor([0, 3], dtype=torch.int64, device="cuda")  # 3 >= len 3
    with pytest.raises(ValueError, match="index out of range"):
        jagged.getitem_jagged_index(off, x, ioff, idx)


@pytest.mark.parametrize("start,stop,step", [(1, None, None), (None, -1, None), (1, None, 2),
                                             (None, None, -1), (-2, 0, -1)])
def test_inner_range_matches_oracle(start, stop, step):
    import torch

    from awkward_gb300 import jagged

    rng = np.random.default_rng(14)
    Lo = rng.poisson(4, 100_000)
    Li = rng.poisson(6, int(Lo.sum()))
    inner = np.concatenate([[0], np.cumsum(Li)]).astype(np.int64)
    x = rng.standard_normal(int(inner[-1])).astype(np.float32)
    nxo, nxc = jagged.inner_range(torch.from_numpy(inner).cuda(), start, stop, step)
    n = len(inner) - 1
    none = jagged.SLICE_NONE
    a = none if start is None else start
    b = none if stop is None else stop
    c = 1 if step is None else step
    lib = oracle.load()
    cl = np.zeros(1, np.int64)
    assert oracle.call(lib, "awkward_ListArray64_getitem_next_range_carrylength", carrylength=cl,
                       fromstarts=inner[:-1].copy(), fromstops=inner[1:].copy(), lenstarts=n,
                       start=a, stop=b, step=c)[0] is None
    e_off = np.zeros(n + 1, np.int64)
    e_carry = np.zeros(max(int(cl[0]), 1), np.int64)
    assert oracle.call(lib, "awkward_ListArray64_getitem_next_range_64", tooffsets=e_off,
                       tocarry=e_carry, fromstarts=inner[:-1].copy(), fromstops=inner[1:].copy(),
                       lenstarts=n, start=a, stop=b, step=c)[0] is None
    np.testing.assert_array_equal(nxo.cpu().numpy(), e_off)
    np.testing.assert_array_equal(nxc.cpu().numpy(), e_carry[: int(cl[0])])
    got = jagged.take(torch.from_numpy(x).cuda(), nxc)
    np.testing.assert_array_equal(got.cpu().numpy(), x[e_carry[: int(cl[0])]])


def test_full_size_chains_properties():
    import torch

    from awkward_gb300 import jagged

    rng, L, off, x, mask = _case(10_000_000, 15)
    d_off = torch.from_numpy(off).cuda()
    d_x = torch.from_numpy(x).cuda()
    d_mask = torch.from_numpy(mask).cuda()
    owner = torch.repeat_interleave(torch.arange(len(L), device="cuda"),
                                    torch.from_numpy(L).cuda())
    # array[mask]: carry = positions of the true entries, offsets = cumulative counts
    ioff, idx = jagged.jagged_mask_to_index(d_off, d_mask)
    too, tocarry = jagged.jagged_apply(d_off, ioff, idx, d_x.numel())
    assert torch.equal(tocarry, torch.nonzero(d_mask).flatten())
    counts = torch.zeros(len(L), dtype=torch.int64, device="cuda").index_add_(
        0, owner, d_mask.to(torch.int64))
    assert torch.equal(too[1:] - too[:-1], counts)
    assert torch.equal(jagged.take(d_x, tocarry), d_x[d_mask])
    # array[idx]: carry = start + (idx mod len)
    ioff_h, idx_h = _index_case(rng, L)
    d_ioff, d_idx = torch.from_numpy(ioff_h).cuda(), torch.from_numpy(idx_h).cuda()
    too2, tocarry2 = jagged.jagged_apply(d_off, d_ioff, d_idx, d_x.numel())
    iowner = torch.repeat_interleave(torch.arange(len(L), device="cuda"),
                                     d_ioff[1:] - d_ioff[:-1])
    Ld = (d_off[1:] - d_off[:-1])[iowner]
    assert torch.equal(tocarry2, d_off[:-1][iowner] + torch.remainder(d_idx, Ld))
    assert torch.equal(too2, d_ioff)
    # two-level [..., 1:]: every inner element but the first
    Lo = rng.poisson(4, 10_000_000)
    Li = rng.poisson(6, int(Lo.sum()))
    inner = torch.from_numpy(np.concatenate([[0], np.cumsum(Li)]).astype(np.int64)).cuda()
    nxo, nxc = jagged.inner_range(inner, 1, None, None)
    keep = torch.ones(int(inner[-1]), dtype=torch.bool, device="cuda")
    starts = inner[:-1][(inner[1:] - inner[:-1]) > 0]
    keep[starts] = False
    assert torch.equal(nxc, torch.nonzero(keep).flatten())
    Lt = torch.from_numpy(Li).cuda()
    assert torch.equal(nxo[1:] - nxo[:-1], torch.clamp(Lt - 1, min=0))


@pytest.mark.parametrize("variant", ["poisson", "base", "all_true", "all_false", "long_list",
                                     "half_empty"])
@pytest.mark.parametrize("dt", [np.uint8, np.int16, np.float32, np.float64])
def test_one_pass_mask_select_equals_the_chain(variant, dt):
    """array[mask] in one pass gives the chain's offsets, carry and content, bit for bit."""
    import torch

    from awkward_gb300 import jagged

    p = {"all_true": 1.0, "all_false": 0.0}.get(variant, 0.4)
    extra = np.array([100_000]) if variant == "long_list" else None
    pe = 0.5 if variant == "half_empty" else 0.01
    _rng, L, off, x, mask = _case(20_000, 7, base=5 if variant == "base" else 0, extra=extra,
                                  p=p, pe=pe)
    xs = (x * 3).astype(dt) if np.dtype(dt).kind != "f" else x.astype(dt)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    doff, dx, dm = d(off), d(xs), d(mask)
    so, sc, scarry = jagged.mask_select(doff, dx, dm, with_carry=True)
    io, idx = jagged.jagged_mask_to_index(doff, dm)
    co, ccarry = jagged.jagged_apply(doff, io, idx, dx.numel())
    cc = jagged.take(dx, ccarry)
    torch.testing.assert_close(so, co, rtol=0, atol=0)
    torch.testing.assert_close(scarry, ccarry, rtol=0, atol=0)
    assert torch.equal(sc.view(torch.uint8), cc.view(torch.uint8))
    so2, sc2 = jagged.mask_select(doff, dx, dm)
    assert torch.equal(so2, so) and torch.equal(sc2.view(torch.uint8), sc.view(torch.uint8))


@pytest.mark.parametrize("n", [0, 1, 5000])
def test_one_pass_mask_select_no_elements(n):
    """No lists, or lists that are all empty: offsets of zeros and no content."""
    import torch

    from awkward_gb300 import jagged

    doff = torch.zeros(n + 1, dtype=torch.int64, device="cuda")
    dx = torch.zeros(0, dtype=torch.float32, device="cuda")
    dm = torch.zeros(0, dtype=torch.bool, device="cuda")
    so, sc, scarry = jagged.mask_select(doff, dx, dm, with_carry=True)
    assert torch.equal(so, torch.zeros(n + 1, dtype=torch.int64, device="cuda"))
    assert sc.numel() == 0 and scarry.numel() == 0


@pytest.mark.parametrize("variant", ["poisson", "base", "long_list", "half_empty"])
@pytest.mark.parametrize("dt", [np.uint8, np.int16, np.float32, np.float64])
def test_one_pass_index_select_equals_the_chain(variant, dt):
    """array[idx] in one pass gives the chain's offsets, carry and content, bit for bit
    (negative indices included)."""
    import torch

    from awkward_gb300 import jagged

    extra = np.array([100_000]) if variant == "long_list" else None
    pe = 0.5 if variant == "half_empty" else 0.01
    rng, L, off, x, _mask = _case(20_000, 9, base=5 if variant == "base" else 0, extra=extra,
                                  pe=pe)
    ioff, idx = _index_case(rng, L)
    xs = (x * 3).astype(dt) if np.dtype(dt).kind != "f" else x.astype(dt)
    d = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    doff, dx, dio, dix = d(off), d(xs), d(ioff), d(idx)
    so, sc, scarry = jagged.index_select(doff, dx, dio, dix, with_carry=True)
    co, ccarry = jagged.jagged_apply(doff, dio, dix, dx.numel())
    cc = jagged.take(dx, ccarry)
    torch.testing.assert_close(so, co, rtol=0, atol=0)
    torch.testing.assert_close(scarry, ccarry, rtol=0, atol=0)
    assert torch.equal(sc.view(torch.uint8), cc.view(torch.uint8))
    so2, sc2 = jagged.index_select(doff, dx, dio, dix)
    assert torch.equal(so2, so) and torch.equal(sc2.view(torch.uint8), sc.view(torch.uint8))


def test_one_pass_index_select_errors_and_empty():
    import torch

    from awkward_gb300 import jagged

    off = torch.tensor([0, 2, 5], dtype=torch.int64, device="cuda")
    x = torch.arange(5, dtype=torch.float32, device="cuda")
    ioff = torch.tensor([0, 1, 2], dtype=torch.int64, device="cuda")
    with pytest.raises(ValueError, match="index out of range"):
        jagged.index_select(off, x, ioff, torch.tensor([0, 3], dtype=torch.int64, device="cuda"))
    so, sc = jagged.index_select(off, x, ioff, torch.tensor([-1, -3], dtype=torch.int64,
                                                            device="cuda"))
    assert so.tolist() == [0, 1, 2] and sc.tolist() == [1.0, 2.0]
    # no lists, and lists with no index entries
    empty = torch.zeros(0, dtype=torch.int64, device="cuda")
    so, sc = jagged.index_select(torch.zeros(1, dtype=torch.int64, device="cuda"), x[:0],
                                 torch.zeros(1, dtype=torch.int64, device="cuda"), empty)
    assert so.tolist() == [0] and sc.numel() == 0
    so, sc = jagged.index_select(off, x, torch.zeros(3, dtype=torch.int64, device="cuda"), empty)
    assert so.tolist() == [0, 0, 0] and sc.numel() == 0
