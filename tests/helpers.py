"""Shared comparison helpers for the parity tests."""
import numpy as np

FIELDS = ("rho", "u", "v", "p")


def rel_l1(a, b):
    """Relative L1 difference sum|a-b| / sum|b| (0 when both are all zero)."""
    den = np.abs(b).sum()
    num = np.abs(a - b).sum()
    return float(num / den) if den > 0 else float(num)


def compare_states(got, want, fields=FIELDS):
    return {f: rel_l1(got[f], want[f]) for f in fields}
