"""Golden values of the TT-SVD round at the benchmark's core shapes.

Runs the FP64 oracle (oracle/tt_fp64.py: raw MPO x MPS product, left QR sweep,
right-to-left SVDs) on seeded chains whose cores have the benchmark's shapes
(MPS bond chi = 256, d = 2; MPO bond D = 16, 2 x 2 legs; product bond 4096) and
stores the gauge-invariant results in config2_cores.npz:
  <case>/spectra/<k>  singular values of bond k (descending)
  <case>/discarded    discarded weight per bond
  <case>/xz           <X|Z> as (mantissa, exponent) with <X|Z> = mantissa * 2^exponent
  <case>/zz           <Z|Z> likewise
Inputs are regenerated from the seed by tests (numpy's PCG64 generator gives
the same draws on every platform).  Run from the repository root:
    python tests/golden/make_config2_cores.py
"""
import math
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import tt_fp64 as O  # noqa: E402

CASES = {"n20": (20, 11), "n24": (24, 12)}  # name -> (sites, seed)
CHI, D, DPHYS = 256, 16, 2


def inputs(n, seed):
    rng = np.random.default_rng(seed)
    X = O.random_mps_cores(rng, n, DPHYS, CHI)
    W = O.random_mpo_cores(rng, n, DPHYS, D)
    return X, W


def log2_overlap(A, B):
    """<A|B> as (mantissa, exponent): transfer sweep with power-of-two rescaling."""
    E = np.ones((1, 1))
    expo = 0
    for a, b in zip(A, B):
        T = (E @ b.reshape(b.shape[0], -1)).reshape(a.shape[0] * a.shape[1], b.shape[2])
        E = a.reshape(-1, a.shape[2]).T @ T
        m = float(np.max(np.abs(E)))
        if m > 0:
            e = math.frexp(m)[1]
            E = np.ldexp(E, -e)
            expo += e
    return float(E.reshape(-1)[0]), float(expo)


def main():
    out = {}
    for name, (n, seed) in CASES.items():
        X, W = inputs(n, seed)
        Z, spectra, disc = O.tt_svd_round(O.mpo_mps_product(W, X), CHI)
        out["%s/xz" % name] = np.array(log2_overlap(X, Z))
        out["%s/zz" % name] = np.array(log2_overlap(Z, Z))
        out["%s/discarded" % name] = np.array(disc)
        out["%s/spectra/n" % name] = np.array(len(spectra))
        for k, s in enumerate(spectra):
            out["%s/spectra/%d" % (name, k)] = s
        print(name, "done", flush=True)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "config2_cores.npz"), **out)


if __name__ == "__main__":
    main()
