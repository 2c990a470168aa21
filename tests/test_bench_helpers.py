"""CPU checks of bench.py's host-side helpers: the periodic square lattice of
the reference's own benchmark suite (benchmarks/core_bench.jl:35-63) and the
committed DRAM-traffic figure the headline line reports."""
import importlib.util
from pathlib import Path

import numpy as np
import scipy.sparse as sp

ROOT = Path(__file__).resolve().parents[1]


def _bench():
    spec = importlib.util.spec_from_file_location("bench_module", ROOT / "bench.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_square_lattice_matches_reference_builder():
    b = _bench()
    L = 6
    H, Jx, Jy = b._square_lattice(L)
    Hr = sp.csr_matrix(H)
    # four directed nearest-neighbour entries of -1 per site, no diagonal
    assert np.all(np.diff(Hr.indptr) == 4)
    assert np.all(Hr.data == -1)
    assert abs(Hr.diagonal()).max() == 0
    assert abs(H - H.conj().T).max() == 0
    # site (x, y) -> x + L y; neighbour (x+1, y) carries the current dx = x - xn = -1
    i, j = 0 + L * 0, 1 + L * 0
    assert H[i, j] == -1 and Jx[i, j] == 1 and Jy[i, j] == 0
    # periodic wrap in y: (0, 0) -> (0, L-1) has dy = +1
    j = 0 + L * (L - 1)
    assert H[i, j] == -1 and Jy[i, j] == -1 * 1 and Jx[i, j] == 0
    # the band edge is 4 (normalizeH then rescales by 2*4/(2-0.1))
    assert np.isclose(np.abs(np.linalg.eigvalsh(H.toarray())).max(), 4.0)


def test_committed_traffic_figure_parses():
    b = _bench()
    t = b.profile_traffic("ff")
    assert t is not None and 5e9 < t < 8e9   # bytes per full-size step launch
