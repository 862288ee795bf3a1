"""The asymmetric, non-conformal configuration (96^3-scale convection-
diffusion pair with a 3:2 GGI interface; ``cases.c3``) with the oracle's
GGI overlap weights (test infrastructure).  The product builds the same
weights on the device (mrg_ggi_build, bit-identical to the oracle's)."""
from __future__ import annotations

from multiregionfoam_gb300 import cases


def oracle_weights(fa, fb):
    import oracle as O
    return O.ggi_weights(*fa, *fb)


def c3(scale: int = 1, seed: int = 0, pe_max: float = 10.0, k: float = 1.0, rc: float = 1.0, permute: bool = True):
    return cases.c3(oracle_weights, scale=scale, seed=seed, pe_max=pe_max, k=k, rc=rc, permute=permute)
