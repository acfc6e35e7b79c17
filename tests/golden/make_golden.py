"""Generate the known-answer fixtures that pin the oracle (and the CUDA path).

Each fixture restates a known answer that one of the reference's own tests
checks the imaginary-time bubble / RPA path against (files relative to the
TPRF source tree):

* ``lindhard_square_2orb.npz`` -- test/python/chi00_square_lattice.py:52-141:
  2-orbital square lattice (h_loc, T as at :56-67), n_k = (2, 2, 1), beta = 20,
  mu = 0; the analytic band-basis Lindhard chi00 (lattice/lindhard_chi00.cpp:34-94)
  at nw = 1 and nw = 4.
* ``hubbard_1d_q0.npz`` -- test/python/mean_field.py:212-221,295-351: 1D chain
  t = 1, beta = 5; chi0(q=0, w=0) from the density-of-states integral, and the
  Fazekas RPA value 0.5 chi0 / (1 - U chi0) at U = 6.1.
* ``kanamori_1d_q0.npz`` -- test/python/mean_field_kanamori.py:28-162: 1D chain,
  beta = 0.544; chi0(q=0) from the DOS integral and the closed form
  chi0 / (1 - (U + J) chi0) at U = 2.4, J = 0.6.

The analytic Lindhard arrays are computed by the oracle's restatement of
lindhard_chi00 (a band-basis sum with no FFT and no tail model, independent of
the imaginary-time path); the rest by scipy quadrature. Run:
    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle as O  # noqa: E402


def square_2orb_model():
    h_loc = np.array([[-0.3, -0.5], [-0.5, 0.4]])
    T = -1.0 * np.array([[1.0, 0.23], [0.23, 0.5]])
    return {(0, 0): h_loc, (0, 1): T, (0, -1): T, (1, 0): T, (-1, 0): T}


def main():
    dims = (2, 2, 1)
    beta, mu = 20.0, 0.0
    ek = O.ek_from_hoppings(square_2orb_model(), dims)
    np.savez(os.path.join(HERE, "lindhard_square_2orb.npz"), beta=beta, mu=mu, dims=np.array(dims), e_k=ek,
             chi00_wk_nw1=O.lindhard_chi00(ek, dims, beta, mu, 1),
             chi00_wk_nw4=O.lindhard_chi00(ek, dims, beta, mu, 4))
    t, beta, U = 1.0, 5.0, 6.1
    c0 = O.chi0_q0_integral_1d(t, beta)
    np.savez(os.path.join(HERE, "hubbard_1d_q0.npz"), t=t, beta=beta, U=U, chi0_q0=c0,
             chi_szsz_q0=0.5 * c0 / (1.0 - U * c0))
    beta, U, J = 0.544, 2.4, 0.6
    c0 = O.chi0_q0_integral_1d(t, beta)
    norb = 4
    ueff = U + (norb / 2 - 1) * J
    np.savez(os.path.join(HERE, "kanamori_1d_q0.npz"), t=t, beta=beta, U=U, J=J, chi0_q0=c0,
             chi_szsz_q0=c0 / (1.0 - ueff * c0))
    print("fixtures written to", HERE)


if __name__ == "__main__":
    main()
