"""Wider stencils with one width per field (scafes_wide_*, C ABI) against the
reference's StencilWidthVar run (golden vectors) and the oracle.  The update
is a sum plus one division in the reference's order, so the comparison is
bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import oracle as O
from conftest import load_golden

pytestmark = pytest.mark.gpu


def test_wide_matches_reference_golden(gpu):
    M = gpu
    d = load_golden("stencil_width_var")
    n, T = tuple(int(v) for v in d["n"]), int(d["nsteps"])
    k, j, i = np.meshgrid(*(np.arange(v) for v in n[::-1]), indexing="ij")
    u0 = (i + j + k).astype(np.float64)
    with M.Wide(n, [0, 1, 2]) as w:
        for f in range(3):
            w.upload(f, u0)
        w.step(T)
        for f in range(3):
            assert np.array_equal(w.download(f), d["final"][f]), f


@pytest.mark.parametrize("n,widths", [((19, 13, 11), [3, 1]), ((7, 40, 5), [8, 4, 0]), ((2, 3, 1), [2])])
def test_wide_random_matches_oracle(gpu, n, widths):
    M = gpu
    T = 7
    rng = np.random.default_rng(sum(n))
    g = O.make_grid(n, tau=1.0)
    u0 = [rng.uniform(-1.0, 1.0, (n[2], n[1], n[0])) for _ in widths]
    with M.Wide(n, widths) as w:
        for f, u in enumerate(u0):
            w.upload(f, u)
        w.step(T)
        for f, bw in enumerate(widths):
            assert np.array_equal(w.download(f), O.stencil_width_var(g, u0[f], bw, T)), (f, bw)


def test_wide_errors(gpu):
    M = gpu
    with pytest.raises(M.ScafesError):
        M.Wide((8, 8, 8), [9])
    with pytest.raises(M.ScafesError):
        M.Wide((8, 8, 8), [-1])
    with M.Wide((8, 8, 8), [1]) as w:
        with pytest.raises(M.ScafesError):
            w.upload(1, np.zeros((8, 8, 8)))
        with pytest.raises(M.ScafesError):
            w.upload(0, np.zeros(5))
