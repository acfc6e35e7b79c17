"""FP64 numpy restatement of TPRF's imaginary-time bubble + RPA path.

TEST INFRASTRUCTURE ONLY (the checker for the CUDA path; never shipped or
measured as the product).

Every function cites the reference file:line it restates. Paths are relative
to the TPRF source tree (``c++/triqs_tprf/...``, ``python/triqs_tprf/...``).

Data layout follows TRIQS gf data: mesh indices first, then target indices,
C order, complex128. Momentum / real-space meshes are always 3-dimensional
``dims = (n1, n2, n3)`` (unused dimensions are 1) with the linear index
``(i1 * n2 + i2) * n3 + i3`` and ``k_i = 2*pi*i/n``.
"""
from __future__ import annotations

import itertools
import math
from fractions import Fraction

import numpy as np

__all__ = [
    "fermionic_iw", "bosonic_iw", "tau_points", "default_n_tau",
    "ek_from_hoppings", "kpoints",
    "lattice_dyson_g0_wk", "lattice_dyson_g_wk",
    "fourier_wk_to_wr", "fourier_wr_to_wk",
    "tail_fit_indices", "tail_fit_matrix", "tail_fit",
    "g0_tail_moments_wr",
    "fourier_wr_to_tr", "fit_derivatives", "vandermonde_inverse", "FIT_DERIVATIVE_ROWS",
    "fourier_tr_to_wr", "chi_tr_from_chi_wr", "default_n_iw", "tail_order",
    "bubble_PI_wk", "dynamical_screened_interaction_W", "dynamical_screened_interaction_W_wk",
    "gw_dynamic_sigma", "split_into_dynamic_wk_and_constant_k",
    "chi0_tr_from_grt_PH", "chi_wr_from_chi_tr", "chi_wk_from_chi_wr",
    "chi_wr_from_chi_wk", "chi_trapz_tau", "chi_w0r_from_chi_tr",
    "chi0_w0r_from_grt_PH", "chi0_wr_from_grt_PH",
    "solve_rpa_PH", "imtime_bubble_chi0_wk",
    "lindhard_chi00", "kanamori_charge_and_spin_quartic_interaction_tensors",
    "quartic_tensor_from_charge_and_spin", "kanamori_quartic_tensor",
    "fermi", "chi0_q0_integral_1d",
    "tprf_order_to_matrix_rpa_order", "lose_spin_degree_of_freedom", "rpa_us_tensor", "rpa_uc_tensor",
    "tensor_to_matrix", "matrix_to_tensor", "matrix_rpa", "chi_rpa_spin", "chi_rpa_charge",
    "split_quartic_tensor_in_charge_and_spin", "general_susceptibility_from_charge_and_spin",
    "charge_and_spin_susceptibility_from_general", "hartree_response",
]

# ----------------------------------------------------------------------------
# Meshes (TRIQS imfreq / imtime / brzone conventions)
# ----------------------------------------------------------------------------


def fermionic_iw(beta: float, n_max: int) -> np.ndarray:
    """Full fermionic Matsubara mesh n = -n_max .. n_max-1, i*nu_n = i(2n+1)pi/beta.

    TRIQS ``mesh::imfreq{beta, Fermion, n_max}`` (the mesh every hot-path
    function receives, e.g. ``lattice/gf.cpp:42``).
    """
    n = np.arange(-n_max, n_max)
    return 1j * (2 * n + 1) * np.pi / beta


def bosonic_iw(beta: float, n_iw: int) -> np.ndarray:
    """Full bosonic mesh m = -(n_iw-1) .. n_iw-1, i*omega_m = 2 i m pi / beta.

    TRIQS ``mesh::imfreq{beta, Boson, nw}`` as built by ``make_adjoint_mesh``
    in ``lattice/fourier.hpp:140``.
    """
    m = np.arange(-(n_iw - 1), n_iw)
    return 1j * 2 * m * np.pi / beta


def tau_points(beta: float, n_tau: int) -> np.ndarray:
    """Imaginary-time mesh tau_i = i * beta / (n_tau - 1), i = 0 .. n_tau-1."""
    return np.arange(n_tau) * (beta / (n_tau - 1))


def default_n_tau(n_max: int) -> int:
    """Default time mesh of ``make_adjoint_mesh(imfreq)``: 6 * n_max + 1 points.

    Used by ``fourier_wr_to_tr(g_wr, nt=-1)`` (``lattice/fourier.hpp:107``).
    The value is TRIQS's (not vendored); callers that need certainty pass nt.
    """
    return 6 * n_max + 1


def kpoints(dims) -> np.ndarray:
    """k-vectors (in units of the reciprocal basis, radians) of a brzone mesh, [N_k, 3]."""
    grids = np.meshgrid(*[2 * np.pi * np.arange(n) / n for n in dims], indexing="ij")
    return np.stack([g.ravel() for g in grids], axis=-1)


def ek_from_hoppings(hoppings: dict, dims) -> np.ndarray:
    """Dispersion e(k) = sum_R t(R) exp(i k.R) on a brzone mesh, [N_k, nb, nb].

    Restates ``TBLattice.fourier`` as used by ``python/triqs_tprf/tight_binding.py:27``
    (TRIQS ``tight_binding``): hopping keys are lattice vectors R (1 to 3
    integers), values are nb x nb matrices.
    """
    k = kpoints(dims)
    nb = next(iter(hoppings.values())).shape[0]
    ek = np.zeros((k.shape[0], nb, nb), dtype=complex)
    for R, t in hoppings.items():
        Rv = np.zeros(3)
        Rv[: len(R)] = R
        ek += np.exp(1j * (k @ Rv))[:, None, None] * np.asarray(t, dtype=complex)[None]
    return ek


# ----------------------------------------------------------------------------
# Dyson equation (c++/triqs_tprf/lattice/gf.cpp:42-58, 91-123)
# ----------------------------------------------------------------------------


def lattice_dyson_g0_wk(mu: float, e_k: np.ndarray, beta: float, n_max: int) -> np.ndarray:
    """G0(iv, k) = [(iv + mu) I - e(k)]^-1 per (v, k).  ``lattice/gf.cpp:42-58``."""
    return lattice_dyson_g_wk(mu, e_k, beta, n_max, sigma=None)


def lattice_dyson_g_wk(mu, e_k, beta, n_max, sigma=None) -> np.ndarray:
    """G(iv, k) = [(iv + mu) I - e(k) - Sigma]^-1.  ``lattice/gf.cpp:91-123``.

    ``sigma`` is None, a [N_v, nb, nb] sigma_w or a [N_v, N_k, nb, nb] sigma_wk.
    Output [N_v, N_k, nb, nb].
    """
    nb = e_k.shape[-1]
    iw = fermionic_iw(beta, n_max)
    eye = np.eye(nb)
    m = (iw + mu)[:, None, None, None] * eye - e_k[None]
    if sigma is not None:
        sigma = np.asarray(sigma)
        m = m - (sigma[:, None] if sigma.ndim == 3 else sigma)
    return np.linalg.inv(m)


# ----------------------------------------------------------------------------
# Lattice FFTs (fourier/fourier_lattice.cpp:28-59, fourier/fourier_common.cpp:26-53,
# lattice/fourier.hpp:166-231)
# ----------------------------------------------------------------------------


def fourier_wk_to_wr(g_wk: np.ndarray, dims) -> np.ndarray:
    """k -> r: FFTW_FORWARD (exp(-2 pi i jk/N)) over the k dims, divided by N_k.

    Per frequency slice (``lattice/fourier.hpp:166-197``), plan from
    ``fourier_lattice.cpp:39``, scaling ``fourier_lattice.cpp:49``.
    """
    nw = g_wk.shape[0]
    tgt = g_wk.shape[2:]
    a = g_wk.reshape((nw,) + tuple(dims) + tgt)
    nk = int(np.prod(dims))
    out = np.fft.fftn(a, axes=(1, 2, 3)) / nk
    return out.reshape(g_wk.shape)


def fourier_wr_to_wk(g_wr: np.ndarray, dims) -> np.ndarray:
    """r -> k: FFTW_BACKWARD (exp(+2 pi i jk/N)), no scaling.

    ``lattice/fourier.hpp:200-231``, ``fourier_lattice.cpp:40,55-59``.
    """
    nw = g_wr.shape[0]
    tgt = g_wr.shape[2:]
    a = g_wr.reshape((nw,) + tuple(dims) + tgt)
    nk = int(np.prod(dims))
    out = np.fft.ifftn(a, axes=(1, 2, 3)) * nk
    return out.reshape(g_wr.shape)


chi_wk_from_chi_wr = fourier_wr_to_wk  # lattice/chi_imtime.cpp:289-292
chi_wr_from_chi_wk = fourier_wk_to_wr  # lattice/chi_imtime.cpp:294-297


# ----------------------------------------------------------------------------
# High-frequency tail fit (TRIQS fit_tail; called at fourier/fourier_matsubara.cpp:226)
# ----------------------------------------------------------------------------
#
# PARITY UNPINNED: TRIQS's tail_fitter is not vendored with the reference. This
# is a restatement of its published method -- a linear least-squares fit of
# g(iv) ~ sum_{p=0..P} c_p / (iv)^p on the outer fraction of the mesh, both
# signs of frequency, with the frequencies normalised by omega_max -- with the
# parameters below recorded. Because the fit is linear in the data it is a
# fixed matrix F[p, i] per mesh; the CUDA path applies a matrix built by its
# own host code from the same definition.

TAIL_FRACTION = 0.2
TAIL_N_MAX = 30
TAIL_MAX_ORDER = 9


def tail_fit_indices(n_max: int, statistic: str = "Fermion"):
    """Data indices of the fit points: n_pts on each side of the mesh.

    Fermion (data index n + n_max for n = -n_max .. n_max-1): the positive
    indices 0 .. n_max-1. Boson (data index m + n_max - 1 for m = -(n_max-1) ..
    n_max-1, n_max = nw): the positive indices 1 .. nw-1. Over that range of
    `count` indices, n_pts = round(0.2 count) capped at 30, placed evenly
    (rounded half up) over its top 20 %, mirrored to the negative frequencies.
    """
    if statistic == "Fermion":
        i_min, i_max = 0, n_max - 1
    else:
        i_min, i_max = 1, n_max - 1
    count = i_max - i_min + 1
    n_pts = max(1, min((2 * count + 5) // 10, TAIL_N_MAX))
    n_hi = i_max
    n_lo = min(n_hi, i_min + (8 * count + 5) // 10)
    if n_pts == 1:
        pos = [n_hi]
    else:
        span = n_hi - n_lo
        pos = [n_lo + (2 * j * span + (n_pts - 1)) // (2 * (n_pts - 1)) for j in range(n_pts)]
    if statistic == "Fermion":
        ns = [-n - 1 for n in reversed(pos)] + pos  # Matsubara integers
        return np.array([n + n_max for n in ns], dtype=np.int64)
    ms = [-m for m in reversed(pos)] + pos
    return np.array([m + n_max - 1 for m in ms], dtype=np.int64)


def _omega_max(beta: float, n_max: int, statistic: str) -> float:
    return (2 * n_max - 1) * np.pi / beta if statistic == "Fermion" else 2 * (n_max - 1) * np.pi / beta


def tail_order(beta: float, n_max: int, statistic: str = "Fermion") -> int:
    omega_max = _omega_max(beta, n_max, statistic)
    if omega_max > 1.0:
        order = int(math.floor(16.0 * math.log(10.0) / math.log(omega_max)))
    else:
        order = TAIL_MAX_ORDER
    n_eq = len(tail_fit_indices(n_max, statistic))
    return max(0, min(order, TAIL_MAX_ORDER, n_eq - 1))


def tail_fit_matrix(beta: float, n_max: int, statistic: str = "Fermion"):
    """Return (idx, F, A): moments c = F @ g[idx]; A is the fit design matrix.

    c_p are the coefficients of 1/(iw)^p, p = 0..P. n_max is the fermionic
    n_max or the bosonic nw.
    """
    idx = tail_fit_indices(n_max, statistic)
    P = tail_order(beta, n_max, statistic)
    freqs = fermionic_iw(beta, n_max) if statistic == "Fermion" else bosonic_iw(beta, n_max)
    iw = freqs[idx]
    omega_max = _omega_max(beta, n_max, statistic)
    z = omega_max / iw
    A = z[:, None] ** np.arange(P + 1)[None, :]
    pinv = np.linalg.pinv(A)
    F = (omega_max ** np.arange(P + 1))[:, None] * pinv
    return idx, F, A


def tail_fit(g_w: np.ndarray, beta: float, n_max: int, statistic: str = "Fermion"):
    """Fit moments for every column of g_w [n_freq, ...]. Returns (c [P+1, ...], err)."""
    idx, F, A = tail_fit_matrix(beta, n_max, statistic)
    rest = g_w.shape[1:]
    g = g_w.reshape(g_w.shape[0], -1)[idx]
    c = F @ g
    omega_max = _omega_max(beta, n_max, statistic)
    d = c / (omega_max ** np.arange(c.shape[0]))[:, None]
    err = np.max(np.abs(A @ d - g)) if g.size else 0.0
    return c.reshape((c.shape[0],) + rest), float(err)


def g0_tail_moments_wr(e_k: np.ndarray, mu: float, dims) -> np.ndarray:
    """Exact 1st-3rd moments of G0(iv, r): I delta_r0, (e - mu)(r), (e - mu)^2(r).

    G0(iv, k) = sum_p (e_k - mu)^(p-1) / (iv)^p, transformed k -> r like G.
    Output [3, N_r, nb, nb]. This is the analytic alternative to the fit.
    """
    nb = e_k.shape[-1]
    h = e_k - mu * np.eye(nb)[None]
    m = np.stack([np.broadcast_to(np.eye(nb), h.shape).astype(complex), h, h @ h])
    return fourier_wk_to_wr(m, dims)


# ----------------------------------------------------------------------------
# Matsubara <-> imaginary time (fourier/fourier_matsubara.cpp)
# ----------------------------------------------------------------------------


def _one_fermion(a, b, tau, beta):
    """fourier_matsubara.cpp:31-33."""
    if b >= 0:
        f = np.exp(-b * tau) / (1 + np.exp(-beta * b))
    else:
        f = np.exp(b * (beta - tau)) / (1 + np.exp(beta * b))
    return -a[None, :] * f[:, None]


def _one_boson(a, b, tau, beta):
    """fourier_matsubara.cpp:35-37."""
    if b >= 0:
        f = np.exp(-b * tau) / (np.exp(-beta * b) - 1)
    else:
        f = np.exp(b * (beta - tau)) / (1 - np.exp(b * beta))
    return a[None, :] * f[:, None]


def fourier_wr_to_tr(g_wr, beta, n_tau=-1, moments=None, return_moments=False):
    """G(iv, r) -> G(tau, r), fermionic, per r and target element.

    Restates ``fourier_matsubara.cpp:218-308`` as driven by
    ``lattice/fourier.hpp:99-130``: moments m1..m3 from the tail fit (or
    given), a three-pole model with b = (0, 1, -1) and
    a = (m1-m3, (m2+m3)/2, (m3-m2)/2) is subtracted, the difference scaled by
    1/beta is placed at row (n+L)%L of a length-L array (L = n_tau - 1) and
    FFTW_FORWARD transformed; G(tau) = out * exp(-i pi tau/beta) + model(tau),
    and G[L] = -(G[0] + m1).

    g_wr: [2 n_max, N_r, nb, nb] (any trailing shape). moments: None (fit) or
    [3, N_r, nb, nb] holding m1, m2, m3.
    """
    n_nu = g_wr.shape[0]
    n_max = n_nu // 2
    if n_tau < 0:
        n_tau = default_n_tau(n_max)
    L = n_tau - 1
    if L < 2 * n_max:
        raise RuntimeError("Inverse Fourier: the time mesh must be at least twice as long as the freq mesh")
    rest = g_wr.shape[1:]
    g = g_wr.reshape(n_nu, -1)
    if moments is None:
        c, err = tail_fit(g, beta, n_max)
        if err > 1e-3:
            raise RuntimeError(f"High frequency moments have an error greater than 1e-3: {err}")
        if c.shape[0] < 4:
            raise RuntimeError("Inverse Fourier requires at least a proper 3rd high-frequency moment")
        m1, m2, m3 = c[1], c[2], c[3]
    else:
        mm = np.asarray(moments).reshape(3, -1)
        m1, m2, m3 = mm[0], mm[1], mm[2]
    a1, a2, a3 = m1 - m3, (m2 + m3) / 2, (m3 - m2) / 2
    b1, b2, b3 = 0.0, 1.0, -1.0
    iw = fermionic_iw(beta, n_max)[:, None]
    n = np.arange(-n_max, n_max)
    gin = np.zeros((L, g.shape[1]), dtype=complex)
    gin[(n + L) % L] = (1.0 / beta) * (g - (a1 / (iw - b1) + a2 / (iw - b2) + a3 / (iw - b3)))
    out = np.fft.fft(gin, axis=0)
    tau = tau_points(beta, n_tau)
    gt = np.empty((n_tau, g.shape[1]), dtype=complex)
    t = tau[:L]
    gt[:L] = (out * np.exp(-1j * np.pi * t / beta)[:, None]
              + _one_fermion(a1, b1, t, beta) + _one_fermion(a2, b2, t, beta) + _one_fermion(a3, b3, t, beta))
    gt[L] = -(gt[0] + m1)
    res = gt.reshape((n_tau,) + rest)
    if return_moments:
        return res, np.stack([m1, m2, m3]).reshape((3,) + rest)
    return res


def vandermonde_inverse(order: int = 8) -> np.ndarray:
    """Exact inverse of V[m, j] = m^(j-1), m, j = 1..order, as correctly rounded doubles.

    Row j of the inverse holds the x^j coefficients of the Lagrange basis
    polynomials through the nodes 1..order. ``fourier_matsubara.cpp:56-71``
    hard-codes a floating-point approximation of this same matrix (entries
    off by up to ~6e-10); the exact rationals are used here.
    """
    nodes = list(range(1, order + 1))
    inv = [[Fraction(0)] * order for _ in range(order)]
    for col, m in enumerate(nodes):
        poly = [Fraction(1)]  # coefficients, lowest degree first
        den = Fraction(1)
        for k in nodes:
            if k == m:
                continue
            poly = [Fraction(0)] + poly  # multiply by x
            for i in range(len(poly) - 1):
                poly[i] -= k * poly[i + 1]
            den *= (m - k)
        for j in range(order):
            inv[j][col] = poly[j] / den
    return np.array([[float(v) for v in row] for row in inv])


# Rows 0 and 1 of the inverse Vandermonde table exactly as fourier_matsubara.cpp:56-71
# hard-codes them (the only rows fit_derivatives uses): the reference's own numbers,
# up to ~5e-12 relative from the exact rationals above.
FIT_DERIVATIVE_ROWS = np.array([
    [8.000000000008853, -28.000000000055913, 56.000000000151815, -70.00000000021936,
     56.00000000020795, -28.000000000115904, 8.00000000003683, -1.0000000000049232],
    [-13.742857142879107, 62.10000000013776, -133.5333333337073, 172.75000000055635,
     -141.00000000052023, 71.43333333362274, -20.600000000091182, 2.592857142869304]])
_VINV = FIT_DERIVATIVE_ROWS


def fit_derivatives(gt: np.ndarray, beta: float, statistic: str = "Boson"):
    """Moments m2, m3 of a tau function from 8-point one-sided differences.

    ``fourier_matsubara.cpp:42-97``: d_left[m-1] = (g[m]-g[0])/tau_m,
    d_right[m-1] = (g[N-1]-g[N-1-m])/tau_m, g_vec = Vinv @ d with the
    reference's table rows (FIT_DERIVATIVE_ROWS); m2 = gl0 - s gr0,
    m3 = -(gl1 + s gr1) * 2 / dtau with s = -1 (Fermion) or +1 (Boson).
    gt: [N_tau, ncol]. Returns [2, ncol].
    """
    n = gt.shape[0]
    dtau = beta / (n - 1)
    taus = np.arange(1, 9) * dtau
    d_left = (gt[1:9] - gt[0][None]) / taus[:, None]
    d_right = (gt[n - 1][None] - gt[n - 2 - np.arange(8)]) / taus[:, None]
    gl = _VINV @ d_left
    gr = _VINV @ d_right
    sign = -1.0 if statistic == "Fermion" else 1.0
    m2 = gl[0] - sign * gr[0]
    m3 = -(gl[1] + sign * gr[1]) * 2 / dtau
    return np.stack([m2, m3])


def chi_wr_from_chi_tr(chi_tr: np.ndarray, beta: float, nw: int) -> np.ndarray:
    """Bosonic tau -> i omega per r and element.

    ``lattice/chi_imtime.cpp:279-282`` -> ``lattice/fourier.hpp:133-163`` ->
    ``fourier_matsubara.cpp:123-184``: m1 = -(g[0]-g[L]), m2/m3 from
    ``fit_derivatives``; b = (-1/2, -1, 1), a1 = 4(m1-m3)/3,
    a2 = m3 - (m1+m2)/2, a3 = m1/6 + m2/2 + m3/3; gin[t] = (beta/L)(g(tau_t) -
    model(tau_t)), t < L; FFTW_BACKWARD of length L;
    chi(i w_m) = out[(m+L)%L] + sum_j a_j/(i w_m - b_j).
    """
    n_tau = chi_tr.shape[0]
    L = n_tau - 1
    if L < 2 * nw:
        raise RuntimeError("Fourier: the time mesh must be at least twice as long as the number of positive frequencies")
    rest = chi_tr.shape[1:]
    g = chi_tr.reshape(n_tau, -1)
    m23 = fit_derivatives(g, beta, "Boson")
    m1 = -(g[0] - g[L])
    m2, m3 = m23[0], m23[1]
    b1, b2, b3 = -0.5, -1.0, 1.0
    a1 = 4 * (m1 - m3) / 3
    a2 = m3 - (m1 + m2) / 2
    a3 = m1 / 6 + m2 / 2 + m3 / 3
    tau = tau_points(beta, n_tau)[:L]
    gin = (beta / L) * (g[:L] - (_one_boson(a1, b1, tau, beta) + _one_boson(a2, b2, tau, beta)
                                 + _one_boson(a3, b3, tau, beta)))
    out = np.fft.ifft(gin, axis=0) * L  # FFTW_BACKWARD, unscaled
    m = np.arange(-(nw - 1), nw)
    iw = bosonic_iw(beta, nw)[:, None]
    gw = out[(m + L) % L] + a1 / (iw - b1) + a2 / (iw - b2) + a3 / (iw - b3)
    return gw.reshape((2 * nw - 1,) + rest)


def default_n_iw(n_tau: int) -> int:
    """Frequency count of the adjoint of a time mesh: (n_tau - 1) / 6, the inverse of
    default_n_tau (TRIQS make_adjoint_mesh, recalled; callers can pass it)."""
    return (n_tau - 1) // 6


def fourier_tr_to_wr(g_tr: np.ndarray, beta: float, n_max: int = -1) -> np.ndarray:
    """Fermionic tau -> i nu per r and element (``gf.cpp:257-260`` ->
    ``lattice/fourier.hpp:133-163`` -> ``fourier_matsubara.cpp:123-184``, fermion branch).

    m1 = -(g[0] + g[L]); m2, m3 from ``fit_derivatives`` with the fermion sign;
    b = (0, 1, -1), a = (m1-m3, (m2+m3)/2, (m3-m2)/2); gin[t] = (beta/L)
    exp(i pi tau_t/beta) (g(tau_t) - model(tau_t)) for t < L; FFTW_BACKWARD;
    g(i nu_n) = out[(n+L)%L] + sum_j a_j/(i nu_n - b_j), n = -n_max .. n_max-1.
    """
    n_tau = g_tr.shape[0]
    L = n_tau - 1
    if n_max < 0:
        n_max = default_n_iw(n_tau)
    if L < 2 * n_max:
        raise RuntimeError("Fourier: the time mesh must be at least twice as long as the number of positive frequencies")
    rest = g_tr.shape[1:]
    g = g_tr.reshape(n_tau, -1)
    m23 = fit_derivatives(g, beta, "Fermion")
    m1 = -(g[0] + g[L])
    m2, m3 = m23[0], m23[1]
    b1, b2, b3 = 0.0, 1.0, -1.0
    a1, a2, a3 = m1 - m3, (m2 + m3) / 2, (m3 - m2) / 2
    tau = tau_points(beta, n_tau)[:L]
    model = _one_fermion(a1, b1, tau, beta) + _one_fermion(a2, b2, tau, beta) + _one_fermion(a3, b3, tau, beta)
    gin = (beta / L) * np.exp(1j * np.pi * tau / beta)[:, None] * (g[:L] - model)
    out = np.fft.ifft(gin, axis=0) * L  # FFTW_BACKWARD, unscaled
    n = np.arange(-n_max, n_max)
    iw = fermionic_iw(beta, n_max)[:, None]
    gw = out[(n + L) % L] + a1 / (iw - b1) + a2 / (iw - b2) + a3 / (iw - b3)
    return gw.reshape((2 * n_max,) + rest)


def chi_tr_from_chi_wr(chi_wr: np.ndarray, beta: float, n_tau: int = -1, moments=None) -> np.ndarray:
    """Bosonic i omega -> tau per r and element (``chi_imtime.cpp:284-287`` ->
    ``lattice/fourier.hpp:99-130`` -> ``fourier_matsubara.cpp:218-308``, boson branch).

    Moments m1..m3 from the tail fit on the bosonic mesh (or given); b = (-1/2, -1, 1),
    a1 = 4(m1-m3)/3, a2 = m3-(m1+m2)/2, a3 = m1/6+m2/2+m3/3; the difference
    (1/beta)(chi - model) at row (m+L)%L, FFTW_FORWARD; chi(tau_t) = out[t] +
    sum_j oneBoson(a_j, b_j, tau_t); chi[L] = +(chi[0] + m1).
    """
    nwt = chi_wr.shape[0]
    nw = (nwt + 1) // 2
    if n_tau < 0:
        n_tau = 6 * nw + 1
    L = n_tau - 1
    if L < 2 * nw:
        raise RuntimeError("Inverse Fourier: the time mesh must be at least twice as long as the freq mesh")
    rest = chi_wr.shape[1:]
    g = chi_wr.reshape(nwt, -1)
    if moments is None:
        c, err = tail_fit(g, beta, nw, "Boson")
        if err > 1e-3:
            raise RuntimeError(f"High frequency moments have an error greater than 1e-3: {err}")
        if c.shape[0] < 4:
            raise RuntimeError("Inverse Fourier requires at least a proper 3rd high-frequency moment")
        m1, m2, m3 = c[1], c[2], c[3]
    else:
        mm = np.asarray(moments).reshape(3, -1)
        m1, m2, m3 = mm[0], mm[1], mm[2]
    b1, b2, b3 = -0.5, -1.0, 1.0
    a1 = 4 * (m1 - m3) / 3
    a2 = m3 - (m1 + m2) / 2
    a3 = m1 / 6 + m2 / 2 + m3 / 3
    iw = bosonic_iw(beta, nw)[:, None]
    m = np.arange(-(nw - 1), nw)
    gin = np.zeros((L, g.shape[1]), dtype=complex)
    gin[(m + L) % L] = (1.0 / beta) * (g - (a1 / (iw - b1) + a2 / (iw - b2) + a3 / (iw - b3)))
    out = np.fft.fft(gin, axis=0)
    tau = tau_points(beta, n_tau)[:L]
    gt = np.empty((n_tau, g.shape[1]), dtype=complex)
    gt[:L] = out + _one_boson(a1, b1, tau, beta) + _one_boson(a2, b2, tau, beta) + _one_boson(a3, b3, tau, beta)
    gt[L] = gt[0] + m1
    return gt.reshape((n_tau,) + rest)


# ----------------------------------------------------------------------------
# Bubble (lattice/chi_imtime.cpp:88-136, 139-247)
# ----------------------------------------------------------------------------


def _minus_r(g: np.ndarray, dims) -> np.ndarray:
    """g[..., r, ...] -> g[..., -r mod dims, ...] along axis 1 (the r axis)."""
    n0 = g.shape[0]
    tgt = g.shape[2:]
    a = g.reshape((n0,) + tuple(dims) + tgt)
    a = np.roll(np.flip(a, axis=(1, 2, 3)), 1, axis=(1, 2, 3))
    return a.reshape(g.shape)


def chi0_tr_from_grt_PH(g_tr: np.ndarray, dims) -> np.ndarray:
    """chi0_abcd(tau_i, r) = G_da(tau_i, r) G_bc(beta - tau_i, -r).

    ``lattice/chi_imtime.cpp:88-136`` (the product at ``:127``); beta - tau_i
    is the mesh point N_tau-1-i and -r wraps periodically.
    g_tr: [N_tau, N_r, nb, nb] -> [N_tau, N_r, nb, nb, nb, nb].
    """
    g_m = _minus_r(g_tr, dims)[::-1]
    return np.einsum("trda,trbc->trabcd", g_tr, g_m)


def chi_trapz_tau(chi_t: np.ndarray, beta: float) -> np.ndarray:
    """Trapezoid integral over tau of chi_t [N_tau, ...]. ``chi_imtime.cpp:230-247``."""
    n = chi_t.shape[0]
    s = chi_t.sum(axis=0) - 0.5 * chi_t[0] - 0.5 * chi_t[n - 1]
    return s * (beta / (n - 1))


def chi_w0r_from_chi_tr(chi_tr, beta):
    """Static chi(w=0, r) by trapezoid integration. ``chi_imtime.cpp:250-276``. -> [1, N_r, ...]."""
    return chi_trapz_tau(chi_tr, beta)[None]


def chi0_w0r_from_grt_PH(g_tr, beta, dims):
    """Bubble + trapezoid per r. ``chi_imtime.cpp:185-228``. -> [1, N_r, nb^4]."""
    chi = chi0_tr_from_grt_PH(g_tr, dims)
    return chi_trapz_tau(chi, beta)[None]


def chi0_wr_from_grt_PH(g_tr, beta, dims, nw):
    """Save-memory branch: bubble then tau -> w per r. ``chi_imtime.cpp:139-182``."""
    return chi_wr_from_chi_tr(chi0_tr_from_grt_PH(g_tr, dims), beta, nw)


# ----------------------------------------------------------------------------
# RPA (lattice/rpa.cpp:29-64)
# ----------------------------------------------------------------------------


def _ph_group(x: np.ndarray) -> np.ndarray:
    """[..., a, b, c, d] -> [..., (a b), (d c)] (``rpa.cpp:40,54-55``)."""
    nb = x.shape[-1]
    return np.swapaxes(x, -1, -2).reshape(x.shape[:-4] + (nb * nb, nb * nb))


def _ph_ungroup(m: np.ndarray, nb: int) -> np.ndarray:
    return np.swapaxes(m.reshape(m.shape[:-2] + (nb, nb, nb, nb)), -1, -2)


def solve_rpa_PH(chi0: np.ndarray, U: np.ndarray) -> np.ndarray:
    """chi = [I - chi0 U]^-1 chi0 on PH-grouped nb^2 x nb^2 matrices, per point.

    ``lattice/rpa.cpp:29-64``: rows (a,b), columns (d,c) for both chi0 and U.
    """
    nb = U.shape[0]
    Um = _ph_group(np.asarray(U, dtype=complex))
    c0 = _ph_group(chi0)
    eye = np.eye(nb * nb)
    chi = np.linalg.solve(eye - c0 @ Um, c0)
    return _ph_ungroup(chi, nb)


# ----------------------------------------------------------------------------
# Python driver (python/triqs_tprf/lattice_utils.py:191-269)
# ----------------------------------------------------------------------------


def imtime_bubble_chi0_wk(g_wk, beta, dims, nw=1, save_memory=False, n_tau=-1, moments=None):
    """g_wk -> chi0_wk following ``lattice_utils.py:241-266``."""
    g_wr = fourier_wk_to_wr(g_wk, dims)
    g_tr = fourier_wr_to_tr(g_wr, beta, n_tau, moments=moments)
    if nw == 1:
        chi0_wr = chi0_w0r_from_grt_PH(g_tr, beta, dims)
    elif not save_memory:
        chi0_wr = chi_wr_from_chi_tr(chi0_tr_from_grt_PH(g_tr, dims), beta, nw)
    else:
        chi0_wr = chi0_wr_from_grt_PH(g_tr, beta, dims, nw)
    return chi_wk_from_chi_wr(chi0_wr, dims)


# ----------------------------------------------------------------------------
# GW consumers of the chain (python/triqs_tprf/gw.py, lattice/gw.cpp,
# lattice/dynamical_screened_interaction.cpp, lattice/lattice_utility.cpp)
# ----------------------------------------------------------------------------


def bubble_PI_wk(g_wk, beta, dims):
    """``gw.py:56-91``: the imaginary-time bubble with nw = n_max bosonic frequencies."""
    return imtime_bubble_chi0_wk(g_wk, beta, dims, nw=g_wk.shape[0] // 2)


def dynamical_screened_interaction_W(PI_wk, V_k):
    """W(iw, k) for a static V(k): ``dynamical_screened_interaction.cpp:85-124``.

    denom(a,b,c,d) = delta_ad delta_bc - sum_ef PI(a,b,e,f) V(e,f,c,d) (the
    identity of the PH-grouped view, the natural (e,f) contraction); inverted
    in the PH grouping; W(a,b,c,d) = sum_ef V(a,b,e,f) inv(e,f,c,d).
    PI_wk [n_w, N_k, nb, nb, nb, nb], V_k [N_k, nb, nb, nb, nb].
    """
    nb = V_k.shape[-1]
    eye = np.einsum("ad,bc->abcd", np.eye(nb), np.eye(nb))
    denom = eye[None, None] - np.einsum("wkabef,kefcd->wkabcd", PI_wk, V_k)
    inv = _ph_ungroup(np.linalg.inv(_ph_group(denom)), nb)
    return np.einsum("kabef,wkefcd->wkabcd", V_k, inv)


def dynamical_screened_interaction_W_wk(PI_wk, V_wk):
    """W(iw, k) for a dynamic V(iw, k): ``dynamical_screened_interaction.cpp:30-80``
    (W = V [I - PI V]^-1 on PH-grouped matrices)."""
    nb = V_wk.shape[-1]
    P, V = _ph_group(PI_wk), _ph_group(V_wk)
    return _ph_ungroup(V @ np.linalg.inv(np.eye(nb * nb) - P @ V), nb)


def gw_dynamic_sigma(W_tr, g_tr):
    """``gw.cpp:66-84``: sigma_ab(tau, r) = - sum_cd W_acdb(tau, r) G_cd(tau, r)."""
    return -np.einsum("tracdb,trcd->trab", W_tr, g_tr)


def split_into_dynamic_wk_and_constant_k(chi_wk, beta):
    """``lattice_utility.cpp:57-85``: chi_const(k) = the constant (0th) moment of the
    tail fit of chi(iw, k) on the bosonic mesh; chi_dyn = chi - chi_const."""
    nwt = chi_wk.shape[0]
    nw = (nwt + 1) // 2
    c, _ = tail_fit(chi_wk, beta, nw, "Boson")
    const = c[0]
    return chi_wk - const[None], const


# ----------------------------------------------------------------------------
# Known-answer helpers
# ----------------------------------------------------------------------------


def fermi(x):
    """1 / (exp(x) + 1), as ``lattice_utility`` uses it in ``lindhard_chi00.cpp:61``."""
    return 0.5 * (1.0 - np.tanh(0.5 * np.asarray(x, dtype=float)))


def lindhard_chi00(e_k: np.ndarray, dims, beta: float, mu: float, nw: int) -> np.ndarray:
    """Analytic band-basis bubble chi00(i w_m, q). ``lattice/lindhard_chi00.cpp:34-94``.

    chi_abcd(w, q) = 1/N_k sum_k sum_ij U_k[a,i] U_k^*[d,i] U_{k+q}[c,j] U_{k+q}^*[b,j]
                     (f(e_ki) - f(e_k+q,j)) / (i w + e_k+q,j - e_ki),
    with the w = 0, degenerate limit beta / (4 cosh^2(beta e_ki / 2)).
    """
    nk = e_k.shape[0]
    nb = e_k.shape[-1]
    ek, Uk = np.linalg.eigh(e_k - mu * np.eye(nb)[None])
    iw = bosonic_iw(beta, nw)
    idx = np.arange(nk).reshape(dims)
    chi = np.zeros((len(iw), nk, nb, nb, nb, nb), dtype=complex)
    fk = fermi(beta * ek)
    for q in range(nk):
        qi = np.unravel_index(q, dims)
        kq = np.roll(idx, shift=tuple(-s for s in qi), axis=(0, 1, 2)).ravel()  # index of k+q
        ekq, Ukq, fkq = ek[kq], Uk[kq], fk[kq]
        de = ekq[:, None, :] - ek[:, :, None]  # [k, i, j]
        dn = fk[:, :, None] - fkq[:, None, :]
        A = np.einsum("kai,kdi->kiad", Uk, Uk.conj())
        B = np.einsum("kcj,kbj->kjbc", Ukq, Ukq.conj())
        for wi, w in enumerate(iw):
            with np.errstate(divide="ignore", invalid="ignore"):
                fac = dn / (w + de)
            if abs(w) < 1e-10:
                deg = np.abs(de) < 1e-10
                cosh = np.cosh(0.5 * beta * ek)[:, :, None]
                lim = beta / (4.0 * cosh * cosh)
                fac = np.where(deg, np.broadcast_to(lim, fac.shape), fac)
            chi[wi, q] = np.einsum("kij,kiad,kjbc->abcd", fac, A, B) / nk
    return chi


def chi0_q0_integral_1d(t: float, beta: float) -> float:
    """chi0(q=0, w=0) of the 1D chain from its density of states.

    ``test/python/mean_field.py:212-221`` (with the DOS at ``:176-178`` and
    df/de at ``:123-124``).
    """
    from scipy.integrate import quad

    def integrand(eps):
        rho = 1.0 / np.sqrt(1.0 - (eps / (2 * t)) ** 2) / (2 * t * np.pi)
        df = -beta / 4.0 / np.cosh(0.5 * beta * eps) ** 2
        return -rho * df

    val, _ = quad(integrand, -2.0 * t, 2.0 * t)
    return val


def kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp):
    """Kanamori U_c, U_s in PH order. ``python/triqs_tprf/rpa_tensor.py:87-120``."""
    shape = [norb] * 4
    U_c = np.zeros(shape, dtype=complex)
    U_s = np.zeros(shape, dtype=complex)
    for a, abar, b, bbar in itertools.product(range(norb), repeat=4):
        sc = ss = 0
        if a == abar == b == bbar:
            sc, ss = U, U
        if a == bbar and a != b and abar == b:
            sc, ss = -Up + 2 * J, Up
        if a == abar and a != b and b == bbar:
            sc, ss = 2 * Up - J, J
        if a == b and a != abar and abar == bbar:
            sc, ss = Jp, Jp
        U_c[a, abar, b, bbar] = sc
        U_s[a, abar, b, bbar] = ss
    return U_c, U_s


def quartic_tensor_from_charge_and_spin(U_c, U_s):
    """Spin-resolved (spin slow) tensor from charge/spin parts. ``rpa_tensor.py:175-195``."""
    shape_4 = U_c.shape
    U_8 = np.zeros([2] * 4 + list(shape_4), dtype=U_c.dtype)
    U_uu = -0.5 * (U_c - U_s)
    U_ud = +0.5 * (U_c + U_s)
    for s1, s2 in itertools.product(range(2), repeat=2):
        if s1 == s2:
            U_8[s1, s1, s1, s1] = U_uu
        else:
            U_8[s1, s1, s2, s2] = -U_ud
            U_8[s1, s2, s2, s1] = U_s
    U_8 = np.transpose(U_8, (0, 4, 1, 5, 2, 6, 3, 7))
    return U_8.reshape(2 * np.array(shape_4))


def kanamori_quartic_tensor(norb, U, Up, J, Jp):
    """``rpa_tensor.py:198-233``."""
    U_c, U_s = kanamori_charge_and_spin_quartic_interaction_tensors(norb, U, Up, J, Jp)
    return quartic_tensor_from_charge_and_spin(U_c, U_s)


# ---------------------------------------------------------------------------
# Matrix RPA and the charge / spin channels (known answers of
# test/python/compare_general_rpa_to_matrix_rpa.py:150-241)

def tprf_order_to_matrix_rpa_order(x: np.ndarray) -> np.ndarray:
    """Swap the last two target indices. ``python/triqs_tprf/matrix_rpa.py:42-48``."""
    return np.swapaxes(x, -1, -2)


def lose_spin_degree_of_freedom(x: np.ndarray, rank: int, spin_fast: bool = True) -> np.ndarray:
    """One spin block of the last `rank` (spin, orbital) indices: every second index
    (spin fast) or the second half (spin slow). ``matrix_rpa.py:51-76``, ``rpa_tensor.py:236-256``."""
    norb = x.shape[-1] // 2
    sl = slice(None, None, 2) if spin_fast else slice(norb, None)
    return x[(Ellipsis,) + (sl,) * rank]


def _kanamori_pattern(norb, v_diag, v_pair, v_dens, v_flip):
    """The four Kanamori index patterns of ``matrix_rpa.py:79-142``: a=b=c=d, a=c!=b=d,
    a=b!=c=d, a=d!=b=c, in the cc^+c^+c order of the matrix formalism."""
    out = np.zeros([norb] * 4, dtype=complex)
    for a, b, c, d in itertools.product(range(norb), repeat=4):
        if a == b == c == d:
            out[a, b, c, d] = v_diag
        elif a == c != b == d:
            out[a, b, c, d] = v_pair
        elif a == b != c == d:
            out[a, b, c, d] = v_dens
        elif a == d != b == c:
            out[a, b, c, d] = v_flip
    return out


def rpa_us_tensor(norb, U, Up, J, Jp):
    """Spin-channel vertex of the matrix formalism. ``matrix_rpa.py:79-109``."""
    return _kanamori_pattern(norb, U, Up, J, Jp)


def rpa_uc_tensor(norb, U, Up, J, Jp):
    """Charge-channel vertex of the matrix formalism. ``matrix_rpa.py:112-142``."""
    return _kanamori_pattern(norb, U, -Up + 2 * J, 2 * Up - J, Jp)


def _matrix_rpa_order(norb: int) -> np.ndarray:
    """Row/column order of the matrix formalism: the pairs (a, a) first, then the
    others ascending. ``matrix_rpa.py:145-191``."""
    idx = list(range(norb * norb))
    diag = idx[:: norb + 1]
    return np.array(diag + sorted(set(idx) - set(diag)))


def tensor_to_matrix(x: np.ndarray) -> np.ndarray:
    norb = x.shape[-1]
    o = _matrix_rpa_order(norb)
    m = x.reshape(x.shape[:-4] + (norb * norb, norb * norb))
    return m[..., o, :][..., :, o]


def matrix_to_tensor(m: np.ndarray) -> np.ndarray:
    norb = int(round(np.sqrt(m.shape[-1])))
    inv = np.argsort(_matrix_rpa_order(norb))
    return m[..., inv, :][..., :, inv].reshape(m.shape[:-2] + (norb,) * 4)


def matrix_rpa(chi0_m: np.ndarray, u_m: np.ndarray) -> np.ndarray:
    """[1 - chi0 u]^-1 chi0 on matrices. ``matrix_rpa.py:194-212``."""
    n = chi0_m.shape[-1]
    return np.linalg.solve(np.eye(n) - chi0_m @ u_m, chi0_m)


def chi_rpa_spin(chi0: np.ndarray, us: np.ndarray) -> np.ndarray:
    """``matrix_rpa.py:215-234``."""
    return matrix_to_tensor(matrix_rpa(tensor_to_matrix(chi0), tensor_to_matrix(us)))


def chi_rpa_charge(chi0: np.ndarray, uc: np.ndarray) -> np.ndarray:
    """With -uc (the charge channel's sign). ``matrix_rpa.py:237-257``."""
    return matrix_to_tensor(matrix_rpa(tensor_to_matrix(chi0), -tensor_to_matrix(uc)))


def split_quartic_tensor_in_charge_and_spin(U_4: np.ndarray):
    """(U_c, U_s) of a spin-slow quartic tensor: U_c = -U_uuuu - U_uudd,
    U_s = U_uuuu - U_uudd, after checking that spin is conserved.
    ``python/triqs_tprf/rpa_tensor.py:123-172``."""
    n = U_4.shape[0] // 2
    U_8 = U_4.reshape(2, n, 2, n, 2, n, 2, n).transpose(0, 2, 4, 6, 1, 3, 5, 7)
    for s in itertools.product(range(2), repeat=4):
        conserving = (s[0] == s[1] and s[2] == s[3]) or (s[0] == s[3] and s[1] == s[2])
        if not conserving:
            np.testing.assert_array_almost_equal(U_8[s], 0.0)
    return -U_8[0, 0, 0, 0] - U_8[0, 0, 1, 1], U_8[0, 0, 0, 0] - U_8[0, 0, 1, 1]


def _spin_slices(norb, spin_fast):
    return (slice(None, None, 2), slice(1, None, 2)) if spin_fast else (slice(norb), slice(norb, None))


def general_susceptibility_from_charge_and_spin(chi_c, chi_s, spin_fast=True):
    """chi_uuuu = chi_dddd = (chi_c + chi_s)/2, chi_uudd = chi_dduu = (chi_c - chi_s)/2,
    chi_uddu = chi_duud = chi_s. ``rpa_tensor.py:259-299``."""
    norb = chi_c.shape[-1]
    out = np.zeros(chi_c.shape[:-4] + (2 * norb,) * 4, dtype=complex)
    up, dn = _spin_slices(norb, spin_fast)
    e = (Ellipsis,)
    out[e + (up, up, up, up)] = out[e + (dn, dn, dn, dn)] = 0.5 * (chi_c + chi_s)
    out[e + (up, up, dn, dn)] = out[e + (dn, dn, up, up)] = 0.5 * (chi_c - chi_s)
    out[e + (up, dn, dn, up)] = out[e + (dn, up, up, dn)] = chi_s
    return out


def charge_and_spin_susceptibility_from_general(chi, spin_fast=True):
    """(chi_c, chi_s) = (chi_uuuu + chi_uudd, chi_uuuu - chi_uudd). ``rpa_tensor.py:302-340``."""
    norb = chi.shape[-1] // 2
    up, dn = _spin_slices(norb, spin_fast)
    e = (Ellipsis,)
    return chi[e + (up, up, up, up)] + chi[e + (up, up, dn, dn)], chi[e + (up, up, up, up)] - chi[e + (up, up, dn, dn)]


# ---------------------------------------------------------------------------
# Hartree linear response (known answer of test/python/hartree_response.py:123-176)

def hartree_response(e_k: np.ndarray, beta: float, mu: float, U_abcd: np.ndarray, eps: float = 1e-9):
    """Static uniform response of the mean-field (Hartree) lattice to a density field,
    by central differences of the density matrix, as
    ``python/triqs_tprf/hf_response.py:56-86, 254-290`` computes it:
    chi0_ab = -(1/N_k) sum_k d rho_k,bb / d F_aa (field F_aa on orbital a, step eps)
    and chi_ab = chi0 [1 - U_ab chi0]^-1 with U_ab = U_abcd[a, a, b, b]."""
    nk, nb = e_k.shape[0], e_k.shape[-1]
    E = e_k - mu * np.eye(nb)

    def rho(H):
        w, v = np.linalg.eigh(H)
        f = 1.0 / (np.exp(beta * w) + 1.0)
        return np.einsum("kab,kb,kcb->kac", v, f, v.conj())

    chi0 = np.zeros((nb, nb), dtype=complex)
    for a in range(nb):
        F = np.zeros((nb, nb))
        F[a, a] = 1.0
        d = (rho(E + eps * F) - rho(E - eps * F)).sum(axis=0) / (2.0 * eps * nk)
        chi0[a] = -np.diag(d)
    U_ab = np.array([[U_abcd[a, a, b, b] for b in range(nb)] for a in range(nb)])
    chi = chi0 @ np.linalg.inv(np.eye(nb) - U_ab @ chi0)
    return chi0, chi
