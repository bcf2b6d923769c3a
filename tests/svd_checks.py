"""Comparisons for the truncation step (tensor_su2::svd) shared by the CPU
oracle tests and the GPU parity tests.

The per-sector factors come from a Gram-matrix eigendecomposition
(tensor.cpp:1488-1541): a singular value s is known to about eps*s_max^2/s and
each column only up to its sign (and a rotation inside a degenerate set), so
the checks compare what is independent of that gauge."""
import numpy as np


def svd_value_tolerance(ref, smax):
    """1e-12*s_max plus the Gram method's eps*s_max^2/s."""
    return 1e-12 * smax + 1e-15 * smax**2 / np.maximum(np.abs(ref), 1e-300)


def check_truncation_values(wout, ref, nkept):
    """The kept values (the first nkept of wout, the reference's order) within
    svd_value_tolerance; of the discarded tail only the values above 1e-6 of
    the largest are compared (as a sorted set): below that the Gram
    eigenvalues are rounding noise, and the reference keeps every positive one
    above 1e-100 of the largest (tensor.cpp:1534-1541), so even their number
    is noise."""
    wout = np.asarray(wout)
    smax = np.abs(ref).max()
    assert len(wout) >= nkept
    assert np.all(np.abs(wout[:nkept] - ref[:nkept]) <= svd_value_tolerance(ref[:nkept], smax))
    floor = 1e-6 * smax
    a = np.sort(wout[nkept:][wout[nkept:] > floor])
    b = np.sort(ref[nkept:][ref[nkept:] > floor])
    assert len(a) == len(b)
    assert np.all(np.abs(a - b) <= svd_value_tolerance(b, smax))


def check_mps(oracle, tu, tv, rtu, rtv, tol=1e-10):
    """tu, tv (Struct, x) against the reference's rtu, rtv: the same
    structure and blocks, and per kept sector c the gauge-free products
    U_c V_c^T (the kept part of the wave function, relative Frobenius error
    below tol) and the column norms of U_c and V_c (each a power of one
    singular value; compared within tol of the sector's largest)."""
    for (S, x), (R, rx) in ((tu, rtu), (tv, rtv)):
        assert S.desc().tolist() == R.desc().tolist()
        assert np.asarray(S.flag).tolist() == np.asarray(R.flag).tolist()
        assert len(x) == len(rx)
    U, V = oracle.mps_sector_matrices(*tu), oracle.mps_sector_matrices(*tv)
    RU, RV = oracle.mps_sector_matrices(*rtu), oracle.mps_sector_matrices(*rtv)
    assert sorted(U) == sorted(RU)
    for c in RU:
        p, rp = U[c] @ V[c].T, RU[c] @ RV[c].T
        assert np.linalg.norm(p - rp) <= tol * np.linalg.norm(rp), c
        for a, b in ((U[c], RU[c]), (V[c], RV[c])):
            na, nb = np.linalg.norm(a, axis=0), np.linalg.norm(b, axis=0)
            assert np.all(np.abs(na - nb) <= tol * nb.max()), c
