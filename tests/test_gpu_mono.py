"""Monolithic interface coefficients on the GPU (mrg_mono_*) against the
oracle (oracle/mono_oracle.py): k, Tw and the right-hand side bit-identical
on both sides, for a conformal interface with repeated face cells and a
non-conformal 3:2 GGI interface, without and with radiation, and with the
diffusivity clip active."""
import numpy as np
import pytest

import mono_oracle as M
from mono_case import interface

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("conformal,radiation,ratio", [(True, False, 1.0), (True, True, 1.0), (False, False, 1.0),
                                                       (False, True, 1.0), (False, False, 1e4)])
def test_mono_bitexact(mrg, ctx, oracle_mod, conformal, radiation, ratio):
    a, b, F = interface(3, conformal=conformal, oracle_mod=oracle_mod)
    F["f_a"] = F["f_a"] * ratio
    mono = mrg.MonoInterface(ctx, a, b)
    dev = {k: ctx.to_device(np.ascontiguousarray(v, np.float64)) for k, v in F.items()}
    bufs = []
    try:
        for side, (own, nbr, o, n) in enumerate(((a, b, "a", "b"), (b, a, "b", "a"))):
            nf = len(own["face_cells"])
            d_k, d_tw = ctx.dev_alloc(8 * nf), ctx.dev_alloc(8 * nf)
            bufs += [d_k, d_tw]
            qo = dev["Qr_" + o] if radiation else None
            qn = dev["Qr_" + n] if radiation else None
            mono.update(side, dev["T_" + o], dev["T_" + n], dev["f_" + o], dev["f_" + n], qo, qn, d_k, d_tw)
            k = ctx.from_device(d_k, np.empty(nf))
            tw = ctx.from_device(d_tw, np.empty(nf))
            kr, twr = M.update(own, nbr, F["T_" + o], F["T_" + n], F["f_" + o], F["f_" + n],
                               F["Qr_" + o] if radiation else None, F["Qr_" + n] if radiation else None)
            assert k.tobytes() == kr.tobytes() and tw.tobytes() == twr.tobytes(), side
            if ratio > 1.0 and side == 0:
                kOwn = F["f_a"] / (1 - a["w"]) / a["mld"]
                assert np.any(k < kOwn * 0.999)   # the clip is active somewhere
            mono.source(side, dev["T_" + o], dev["T_" + n], d_tw, d_k, dev["f_" + o], dev["b_" + o])
            bg = ctx.from_device(dev["b_" + o], np.empty(own["n_cells"]))
            br = M.source(own, nbr, F["T_" + o], F["T_" + n], twr, kr, F["f_" + o], F["b_" + o])
            assert bg.tobytes() == br.tobytes(), side
    finally:
        for p in list(dev.values()) + bufs:
            ctx.dev_free(p)
        mono.close()


def test_mono_rejects_bad_patches(mrg, ctx):
    a, b, F = interface(4, conformal=True)
    bad = dict(a, w=np.where(np.arange(len(a["w"])) == 3, 1.0, a["w"]))
    with pytest.raises(mrg.MrgError, match="weights"):
        mrg.MonoInterface(ctx, bad, b)
    bad = dict(a, face_cells=np.where(np.arange(len(a["w"])) == 5, a["n_cells"], a["face_cells"]).astype(np.int32))
    with pytest.raises(mrg.MrgError, match="face cell"):
        mrg.MonoInterface(ctx, bad, b)
