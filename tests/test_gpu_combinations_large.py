"""GPU parity of ListArray combinations beyond the golden fixtures.

* Bit-exact against the C oracle on seeded inputs: n = 1, 2, 3, 4, with and
  without replacement, int64 / int32 / uint32 starts and stops, list sizes
  at the edges (0, 1, 2, 3) and up to a few hundred elements, and lists that
  are not contiguous (starts/stops of a ListArray, not offsets).
* At the full C3 size (5,000,000 lists, lengths min(Poisson(6), 40), n = 2)
  the output is checked by properties that pin it completely: per list
  exactly C(L, 2) tuples, every tuple inside its list, and strictly
  increasing in lexicographic order -- the only sequence with those
  properties is the CPU's enumeration.
"""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

NP_OF = {"ListArray64": np.int64, "ListArray32": np.int32, "ListArrayU32": np.uint32}


def _lengths(kind, rng, nl):
    if kind == "poisson6":
        return np.minimum(rng.poisson(6, nl), 40)
    if kind == "poisson4":
        return rng.poisson(4, nl)
    if kind == "edges":
        return np.array([0, 1, 2, 3, 0, 0, 2, 1, 4, 5, 40, 0, 3] * (nl // 13 + 1))[:nl]
    if kind == "wide":
        L = rng.poisson(3, nl)
        L[:: max(nl // 7, 1)] = rng.integers(100, 300, len(L[:: max(nl // 7, 1)]))
        return L
    raise KeyError(kind)


def _starts_stops(L, rng, gaps):
    if not gaps:
        off = np.concatenate([[0], np.cumsum(L)])
        return off[:-1].copy(), off[1:].copy()
    # a ListArray whose lists sit at arbitrary, non-contiguous places
    starts = rng.integers(0, 10_000, len(L))
    return starts, starts + L


def _gpu_combinations(prefix, dt, n, replacement, starts, stops):
    import torch

    import awkward_gb300

    be = awkward_gb300.backend()
    nl = len(starts)
    st = torch.from_numpy(starts.astype(dt)).cuda()
    sp = torch.from_numpy(stops.astype(dt)).cuda()
    tot = torch.empty(1, dtype=torch.int64, device="cuda")
    too = torch.empty(nl + 1, dtype=torch.int64, device="cuda")
    be.by_name(f"awkward_{prefix}_combinations_length_64")(tot, too, n, replacement, st, sp, nl)
    be.synchronize()
    P = int(tot.item())
    rows = [torch.full((max(P, 1),), -5, dtype=torch.int64, device="cuda") for _ in range(n)]
    ti = torch.empty(n, dtype=torch.int64, device="cuda")
    fi = torch.zeros(n, dtype=torch.int64, device="cuda")
    be.by_name(f"awkward_{prefix}_combinations_64")(rows, ti, fi, n, replacement, st, sp, nl)
    be.synchronize()
    return P, too.cpu().numpy(), [r.cpu().numpy()[:P] for r in rows], ti.cpu().numpy()


def _oracle_combinations(prefix, dt, n, replacement, starts, stops):
    lib = oracle.load()
    nl = len(starts)
    tot = np.zeros(1, np.int64)
    too = np.zeros(nl + 1, np.int64)
    s, p = starts.astype(dt), stops.astype(dt)
    assert oracle.call(lib, f"awkward_{prefix}_combinations_length_64", totallen=tot, tooffsets=too,
                       n=n, replacement=replacement, starts=s, stops=p, length=nl)[0] is None
    P = int(tot[0])
    rows = [np.zeros(max(P, 1), np.int64) for _ in range(n)]
    ti = np.zeros(n, np.int64)
    assert oracle.call(lib, f"awkward_{prefix}_combinations_64", tocarry=rows, toindex=ti,
                       fromindex=np.zeros(n, np.int64), n=n, replacement=replacement,
                       starts=s, stops=p, length=nl)[0] is None
    return P, too, [r[:P] for r in rows], ti


CASES = [
    ("poisson6", 200_000, 2, False, False, "ListArray64"),
    ("poisson6", 50_000, 2, True, False, "ListArray64"),
    ("poisson4", 100_000, 3, False, False, "ListArray64"),
    ("poisson4", 40_000, 3, True, True, "ListArray32"),
    ("edges", 20_000, 2, False, True, "ListArrayU32"),
    ("edges", 20_000, 3, False, False, "ListArray64"),
    ("edges", 20_000, 1, False, False, "ListArray64"),
    ("poisson4", 20_000, 4, False, False, "ListArray64"),
    ("poisson4", 10_000, 4, True, False, "ListArray64"),
    ("wide", 3_000, 2, False, False, "ListArray64"),
    ("wide", 1_000, 3, False, True, "ListArray64"),
]


@pytest.mark.parametrize("kind,nl,n,replacement,gaps,prefix", CASES,
                         ids=[f"{c[0]}-{c[1]}-n{c[2]}-{'rep' if c[3] else 'norep'}-"
                              f"{'gaps' if c[4] else 'offsets'}-{c[5]}" for c in CASES])
def test_combinations_match_oracle(kind, nl, n, replacement, gaps, prefix):
    rng = np.random.default_rng(nl + 7 * n + (3 if replacement else 0))
    L = _lengths(kind, rng, nl)
    starts, stops = _starts_stops(L, rng, gaps)
    dt = NP_OF[prefix]
    P, too, rows, ti = _gpu_combinations(prefix, dt, n, replacement, starts, stops)
    eP, etoo, erows, eti = _oracle_combinations(prefix, dt, n, replacement, starts, stops)
    assert P == eP
    np.testing.assert_array_equal(too, etoo)
    np.testing.assert_array_equal(ti, eti)
    for r, e in zip(rows, erows):
        np.testing.assert_array_equal(r, e)


def test_combinations_pairs_full_size_properties():
    import torch

    rng = np.random.default_rng(3)
    nl = 5_000_000
    L = np.minimum(rng.poisson(6, nl), 40)
    starts, stops = _starts_stops(L, rng, False)
    P, too, rows, ti = _gpu_combinations("ListArray64", np.int64, 2, False, starts, stops)
    Lt = torch.from_numpy(L).cuda()
    expect = Lt * (Lt - 1) // 2
    assert P == int(expect.sum().item())
    too_t = torch.from_numpy(too).cuda()
    assert torch.equal(too_t[1:] - too_t[:-1], expect)
    a = torch.from_numpy(rows[0]).cuda()
    b = torch.from_numpy(rows[1]).cuda()
    # list of every slot
    owner = torch.repeat_interleave(torch.arange(nl, device="cuda"), expect)
    st = torch.from_numpy(starts).cuda()[owner]
    sp = torch.from_numpy(stops).cuda()[owner]
    assert bool(((a >= st) & (a < b) & (b < sp)).all())
    same = owner[1:] == owner[:-1]
    inc = (a[1:] > a[:-1]) | ((a[1:] == a[:-1]) & (b[1:] > b[:-1]))
    assert bool(inc[same].all())
    assert ti.tolist() == [P, P]


def test_row_pointer_arrays_are_reused_and_rebuilt():
    """The int64_t** argument's device array is cached by the rows' addresses:
    the same rows reuse it, other rows get their own, and calls through either
    write into the rows they name."""
    import torch

    import awkward_gb300
    from awkward_gb300 import kernel_table

    be = awkward_gb300.backend()
    k = be.by_name("awkward_ListArray64_combinations_64")
    off = torch.tensor([0, 3, 5], dtype=torch.int64, device="cuda")
    st, sp = off[:-1].contiguous(), off[1:].contiguous()
    ti = torch.empty(2, dtype=torch.int64, device="cuda")
    fi = torch.zeros(2, dtype=torch.int64, device="cuda")
    rows_a = [torch.full((4,), -1, dtype=torch.int64, device="cuda") for _ in range(2)]
    rows_b = [torch.full((4,), -1, dtype=torch.int64, device="cuda") for _ in range(2)]
    dev = torch.device("cuda", torch.cuda.current_device())
    k(rows_a, ti, fi, 2, False, st, sp, 2)
    arr = kernel_table._pointer_array(dev, tuple(t.data_ptr() for t in rows_a))
    k(rows_a, ti, fi, 2, False, st, sp, 2)
    assert kernel_table._pointer_array(dev, tuple(t.data_ptr() for t in rows_a)) is arr
    k(rows_b, ti, fi, 2, False, st, sp, 2)
    be.synchronize()
    expect = [[0, 0, 1, 3], [1, 2, 2, 4]]
    assert [r.tolist() for r in rows_a] == expect and [r.tolist() for r in rows_b] == expect
    assert arr.tolist() == [t.data_ptr() for t in rows_a]
