"""Shared helpers of the test suite."""
from __future__ import annotations

import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")
GOLDEN_CASES = ["plain16k", "random3001", "wrap700", "faces512", "onecell40", "single1"]

# Single-step parity bar for velocities and forces: relative error 1e-5,
# measured per particle on the 3-vector, against a floor so that particles
# with (near) zero force are judged on the absolute scale of a typical force.
REL_TOL = 1e-5


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, f"{name}.npz")) as z:
        return {k: z[k] for k in z.files}


def oracle_params(raw: bytes):
    from oracle import oracle as O
    return O.SimParams.from_buffer_copy(bytes(raw))


def product_params(raw: bytes):
    from fullc0ntact_gb300.params import SimParams
    return SimParams.from_buffer_copy(bytes(raw))


def full_cells(g: dict, num_cells: int):
    cs = np.full(num_cells, 0xFFFFFFFF, np.uint32)
    cs[g["cells"]] = g["cell_start"]
    return cs


def rel_err_vec(a: np.ndarray, b: np.ndarray, floor: float) -> np.ndarray:
    """|a - b| / max(|b|, floor) per row of 3-vectors.  Rows where the
    reference is NaN (coincident particles divide by a zero distance, in the
    reference as here) must be NaN in `a` too and count as error 0."""
    a3 = a[:, :3].astype(np.float64)
    b3 = b[:, :3].astype(np.float64)
    na, nb = np.isnan(a3).any(axis=1), np.isnan(b3).any(axis=1)
    assert np.array_equal(na, nb), "NaN rows differ"
    d = np.linalg.norm(np.where(nb[:, None], 0.0, a3 - b3), axis=1)
    s = np.maximum(np.linalg.norm(np.where(nb[:, None], 0.0, b3), axis=1), floor)
    return d / s


def force_floor(forces: np.ndarray) -> float:
    """A force scale: the median magnitude of the nonzero forces (1e-12 if all
    forces vanish)."""
    m = np.linalg.norm(forces[:, :3].astype(np.float64), axis=1)
    m = m[np.isfinite(m) & (m > 0)]
    return float(np.median(m)) if m.size else 1e-12


def check_cell_tables(cs_a, ce_a, cs_b, ce_b):
    """cellStart must agree everywhere; cellEnd where the cell is non-empty
    (the reference leaves cellEnd of empty cells stale)."""
    np.testing.assert_array_equal(cs_a, cs_b)
    ne = cs_b != 0xFFFFFFFF
    np.testing.assert_array_equal(ce_a[ne], ce_b[ne])


def assert_same_floats(a: np.ndarray, b: np.ndarray) -> None:
    """Bitwise equality of float32 arrays, except that any NaN matches any NaN
    (x86-64 and aarch64 produce different NaN bit patterns)."""
    na, nb = np.isnan(a), np.isnan(b)
    np.testing.assert_array_equal(na, nb)
    np.testing.assert_array_equal(np.where(na, 0, a.view(np.uint32)),
                                  np.where(nb, 0, b.view(np.uint32)))
