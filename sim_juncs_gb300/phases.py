"""CEP and envelope extraction of monitor series on the GPU (sj_extract_phases,
sj_extract_monitor_phases): the reference's scripts/phases.py class `signal`
on the path its sweeps take, signal(t, v, lowpass_inc) then get_envelope()
and get_skewness(), batched one thread block per series."""
import ctypes as C

import numpy as np

from . import _abi

FIELDS = ("f0", "phi", "t0_corr", "t0", "mu", "sig", "skew", "f0_ind", "band_lo", "band_hi",
          "lowpass_steps", "status")


def _to_dicts(res):
    out = []
    for r in res:
        d = {k: getattr(r, k) for k in FIELDS}
        d["amp"] = complex(r.amp[0], r.amp[1])
        out.append(d)
    return out


def extract_phases(t, v, lowpass_inc=1.0):
    """Per series of v ([n_series][n_samples], sampled at t) a dict of f0,
    phi (the CEP), t0_corr, t0, amp (the envelope at its peak), mu, sig,
    skew, f0_ind, the band [band_lo, band_hi), lowpass_steps and status
    (_abi.PHASE_*)."""
    lib = _abi.load_library()
    t = np.ascontiguousarray(t, dtype=np.float64)
    v = np.ascontiguousarray(np.atleast_2d(v), dtype=np.float64)
    n, m = v.shape
    assert t.size == m
    res = (_abi.PhaseResult * max(n, 1))()
    _abi.check(lib, lib.sj_extract_phases(n, m, t.ctypes.data_as(C.POINTER(C.c_double)),
                                          v.ctypes.data_as(C.POINTER(C.c_double)), float(lowpass_inc), res))
    return _to_dicts(res[:n])


def monitor_phases(fields, lowpass_inc=1.0):
    """The same for every monitor of every instance of a Fields, read on the
    device; one list per instance."""
    lib = fields.lib
    counts = [sum(1 for p in inst.probes if p.monitor) for inst in fields.instances]
    total = sum(counts)
    res = (_abi.PhaseResult * max(total, 1))()
    fields._ck(lib.sj_extract_monitor_phases(fields.handle, float(lowpass_inc), res, total))
    flat = _to_dicts(res[:total])
    out, off = [], 0
    for c in counts:
        out.append(flat[off:off + c])
        off += c
    return out
