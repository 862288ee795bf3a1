"""CPU restatement of multiRegionFoam's monolithic interface coefficients
(test infrastructure only: tests import it to check the GPU kernels in
multiregionfoam_gb300/csrc/mono.cu).

One side of a regionCouple interface ("own"), its shadow ("nbr"); paths
within the multiRegionFoam repository, under src/fvPatchFields/
coupledFvPatchFields/monolithicCoupledFvPatchFields/.

  interpolation   the shadow's Tc (patch-internal temperature), diffusivity
                  (monolithicBase::forig, monolithicBase/monolithicBase.C:
                  97-122) and Qr are packed and GGI-interpolated onto the own
                  faces in one call (monolithicThermalDiffusivity/
                  monolithicThermalDiffusivityFvPatchScalarField.C:205-244,
                  318-357); the GGI sum runs in weight order from zero
  diffusivity     calcThermalDiffusivity (.C:167-276): harmonic kHarm
                  (.C:258-260), kOwn = fOwn / (1 - w) / |delta|, kNei =
                  fNei / w / |delta| (.C:262-263), k = kOwn (kNei + Qr /
                  stabilise(TcNei - TcOwn, SMALL)) / (deltaCoeffs (kOwn +
                  kNei)) (.C:265-269), clipped to [0.01, 100] kHarm (.C:271-274)
  temperature     calcTemperature (.C:280-394): Tw = (Qr + kOwn TcOwn + kNei
                  TcNei) / (kOwn + kNei) (.C:381)
  source          monolithicTemperature/monolithicTemperatureFvPatchScalar
                  Field.C:205-224: s = korig (Tw - TcOwn) - kw deltaCoeffs
                  (TcNei - TcOwn), korig = forig / (1 - w) / |delta|
                  (monolithicBase.C:125-132); manipulateMatrix (.C:227-244):
                  b[faceCells] += s |Sf| in face order

The harmonic interpolation's weights come from foam-extend's harmonic
scheme (external, not in the reference); they are restated here as the
weights wh with wh fOwn + (1 - wh) fNei = 1 / (w / fOwn + (1 - w) / fNei),
wh = w fNei / (w fNei + (1 - w) fOwn): parity unpinned for kHarm's rounding.
Every operation is one IEEE operation in the order of the reference's
expressions (numpy, no contraction).
"""
from __future__ import annotations

import numpy as np

SMALL = 1e-15   # foam's SMALL (double precision)


def stabilise(s, small):
    """foam's stabilise: s + small where s >= 0, else s - small."""
    return np.where(s >= 0.0, s + small, s - small)


def ggi_interp(ptr, addr, w, vals):
    """dst[i] = sum_k w_ik vals[addr_ik] (rows of vals), weight order from 0."""
    vals = np.asarray(vals, dtype=np.float64)
    out = np.zeros((len(ptr) - 1,) + vals.shape[1:])
    for i in range(len(ptr) - 1):
        acc = np.zeros(vals.shape[1:])
        for k in range(ptr[i], ptr[i + 1]):
            acc = acc + w[k] * vals[addr[k]]
        out[i] = acc
    return out


def _interp(own, nbr, T_nbr, f_nbr, Qr_nbr):
    tc_src = np.asarray(T_nbr, np.float64)[nbr["face_cells"]]
    cols = [tc_src, np.asarray(f_nbr, np.float64), np.asarray(Qr_nbr, np.float64) if Qr_nbr is not None
            else np.zeros(len(tc_src))]
    i = ggi_interp(own["ptr"], own["addr"], own["wts"], np.stack(cols, axis=1))
    return i[:, 0], i[:, 1], i[:, 2]


def update(own, nbr, T_own, T_nbr, f_own, f_nbr, Qr_own=None, Qr_nbr=None):
    """(k, Tw) on the own side's faces."""
    tc, fn, qn = _interp(own, nbr, T_nbr, f_nbr, Qr_nbr)
    tco = np.asarray(T_own, np.float64)[own["face_cells"]]
    fo = np.asarray(f_own, np.float64)
    w, mld, dc = own["w"], own["mld"], own["dc"]
    Qr = np.zeros(len(fo))
    if Qr_own is not None:
        Qr = Qr + np.asarray(Qr_own, np.float64)
    if Qr_nbr is not None:
        Qr = Qr + qn
    a, b = w * fn, (1.0 - w) * fo
    wh = a / (a + b)
    kH = wh * fo + (1.0 - wh) * fn
    kOwn = fo / (1.0 - w) / mld
    kNei = fn / w / mld
    k = kOwn * (kNei + Qr / stabilise(tc - tco, SMALL))
    k = k / (dc * (kOwn + kNei))
    k = np.maximum(np.minimum(k, 100 * kH), 0.01 * kH)
    Tw = (Qr + kOwn * tco + kNei * tc) / (kOwn + kNei)
    return k, Tw


def source(own, nbr, T_own, T_nbr, Tw, kw, f_own, b):
    """b with the own side's interface source added (a copy)."""
    tc = ggi_interp(own["ptr"], own["addr"], own["wts"],
                    np.asarray(T_nbr, np.float64)[nbr["face_cells"]][:, None])[:, 0]
    tco = np.asarray(T_own, np.float64)[own["face_cells"]]
    kd = np.asarray(kw, np.float64) * own["dc"]
    korig = np.asarray(f_own, np.float64) / (1.0 - own["w"]) / own["mld"]
    s = korig * (np.asarray(Tw, np.float64) - tco) - kd * (tc - tco)
    out = np.array(b, dtype=np.float64, copy=True)
    for f, c in enumerate(own["face_cells"]):
        out[c] = out[c] + s[f] * own["sf"][f]
    return out
