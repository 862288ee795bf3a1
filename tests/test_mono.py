"""The monolithic-interface oracle (monolithicThermalDiffusivity /
monolithicTemperature coefficients) on the CPU: identities that follow from
the reference's expressions."""
import numpy as np

import mono_oracle as M
from mono_case import interface


def test_equal_diffusivity_centred_faces_give_the_diffusivity():
    # w = 1/2 and deltaCoeffs = 1/|delta|: kOwn = kNei = 2 f / |delta|, so
    # k = kOwn kNei / (deltaCoeffs (kOwn + kNei)) = f, inside the clip
    a, b, F = interface(0, conformal=True)
    for p in (a, b):
        p["w"] = np.full(len(p["w"]), 0.5)
        p["dc"] = 1.0 / p["mld"]
    f = np.full(len(a["face_cells"]), 7.0)
    k, Tw = M.update(a, b, F["T_a"], F["T_b"], f, f)
    np.testing.assert_allclose(k, 7.0, rtol=1e-13)


def test_wall_temperature_between_the_cells_and_zero_source_without_radiation():
    a, b, F = interface(1, conformal=True)
    k, Tw = M.update(a, b, F["T_a"], F["T_b"], F["f_a"], F["f_b"])
    tco = F["T_a"][a["face_cells"]]
    tcn = F["T_b"][b["face_cells"]]
    assert np.all(Tw >= np.minimum(tco, tcn) - 1e-9) and np.all(Tw <= np.maximum(tco, tcn) + 1e-9)
    # unclipped and without radiation, kOwn (Tw - Tc) equals k deltaCoeffs
    # (Tc_nei - Tc): the source correction vanishes (to round-off)
    kOwn = F["f_a"] / (1 - a["w"]) / a["mld"]
    kNei = F["f_b"] / a["w"] / a["mld"]
    unclipped = np.isclose(k, kOwn * kNei / (a["dc"] * (kOwn + kNei)), rtol=1e-12)
    assert unclipped.mean() > 0.5
    b0 = np.zeros(a["n_cells"])
    out = M.source(a, b, F["T_a"], F["T_b"], Tw, k, F["f_a"], b0)
    clipped_cells = np.unique(a["face_cells"][~unclipped])
    cells = np.setdiff1d(np.unique(a["face_cells"]), clipped_cells)
    scale = np.abs(kOwn).max() * 80.0 * a["sf"].max() * 2
    assert len(cells) > 0 and np.abs(out[cells]).max() <= 1e-12 * scale


def test_clip_bounds_and_radiation(oracle_mod):
    a, b, F = interface(2, conformal=False, oracle_mod=oracle_mod)
    k, Tw = M.update(a, b, F["T_a"], F["T_b"], F["f_a"] * 1e4, F["f_b"], F["Qr_a"], F["Qr_b"])
    assert np.all(np.isfinite(k)) and np.all(np.isfinite(Tw))
    kH_lo = 0.01 * np.minimum(F["f_a"].min() * 1e4, F["f_b"].min())
    assert np.all(k > 0) and k.min() >= kH_lo * 0.999
