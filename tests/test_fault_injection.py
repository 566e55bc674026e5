"""Host-side fault injection switch of the kernel table (no GPU needed)."""

from awkward_gb300.kernel_table import FAULT_ENV, injected_fault

NAME = "awkward_ListArray64_getitem_jagged_apply_64"
FAMILY = "awkward_ListArray_getitem_jagged_apply"


def test_injected_fault_matches_specialization_or_family():
    assert injected_fault(NAME, FAMILY, {FAULT_ENV: f"{NAME}:4"}) == 4
    assert injected_fault(NAME, FAMILY, {FAULT_ENV: f"{FAMILY}:32"}) == 32
    assert injected_fault("awkward_reduce_sum_int64_int64_64", "awkward_reduce_sum",
                          {FAULT_ENV: f"{FAMILY}:4"}) is None


def test_injected_fault_ignores_malformed_values():
    for v in ("", NAME, f"{NAME}:", f"{NAME}:x", f"{NAME}:256", f"{NAME}:-1"):
        assert injected_fault(NAME, FAMILY, {FAULT_ENV: v}) is None
    assert injected_fault(NAME, FAMILY, {}) is None
