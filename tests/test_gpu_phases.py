"""CEP/envelope extraction on the device against the reference's own
`signal` (scripts/phases.py:94-450), through the C ABI.

tests/golden/phases_reference.json holds what the reference returns on 12
seeded sweep-like pulses and the 8 gap monitors of the 64^3 junction, and how
far its own answers move when the input moves by 1e-15 relative.  Bar:
  * f0's bin, the band and the low-pass strength exactly; f0 to 1e-12;
  * phi (the CEP) and t0_corr to 1e-11, or to ten times the reference's own
    movement where its phase fit sits on near-zero bins (the synthetic pulses,
    whose carrier is near the sampling's Nyquist frequency);
  * the envelope's peak, mean, width and skewness to 1e-5 relative, or twenty
    times the reference's own movement: its curve_fit stops within its
    tolerance of the least-squares optimum that the kernel solves for;
  * where the reference raises (fewer than five band bins for its phase fit),
    SJ_PHASE_NARROW_BAND with the same f0 and band.
"""
import json
import os

import numpy as np
import pytest

from sim_juncs_gb300 import _abi
from sim_juncs_gb300.phases import extract_phases, monitor_phases

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "phases_reference.json")
LOWPASS_INC = 2.0   # as the generator called the reference


@pytest.fixture(scope="module")
def golden():
    with open(GOLDEN) as fh:
        return json.load(fh)["series"]


def test_phases_match_the_reference(lib, golden):
    by_len = {}
    for i, s in enumerate(golden):
        by_len.setdefault(len(s["t"]), []).append(i)
    got = {}
    for n, idx in by_len.items():
        t = np.asarray(golden[idx[0]]["t"])
        for i in idx:
            assert np.array_equal(np.asarray(golden[i]["t"]), t)
        res = extract_phases(t, np.asarray([golden[i]["v"] for i in idx]), LOWPASS_INC)
        got.update(zip(idx, res))
    for i, s in enumerate(golden):
        r, g = s["reference"], got[i]
        if "error" in r:
            assert r["error"] == "TypeError"
            assert g["status"] == _abi.PHASE_NARROW_BAND, (i, g["status"])
            assert g["band_hi"] - g["band_lo"] < 5
            continue
        assert g["status"] == _abi.PHASE_OK, (i, g["status"])
        sens = s["sensitivity"]
        assert g["f0_ind"] == r["f0_ind"], i
        assert [g["band_lo"], g["band_hi"]] == r["band"], i
        assert g["lowpass_steps"] * LOWPASS_INC == r["lowpass_strength"], i
        assert abs(g["f0"] - r["f0"]) <= 1e-12 * abs(r["f0"]), i
        for k in ("phi", "t0_corr"):
            assert abs(g[k] - r[k]) <= max(1e-11 * max(1.0, abs(r[k])), 10 * sens[k]), (i, k, g[k], r[k])
        env = {"amp": (g["amp"], complex(*r["amp"])), "mu": (g["mu"], r["mu"]), "sig": (g["sig"], r["sig"]),
               "skew": (g["skew"], r["skew"])}
        for k, (a, b) in env.items():
            assert abs(a - b) <= max(1e-5 * abs(b), 20 * sens[k]), (i, k, a, b)


def test_monitor_phases_read_on_the_device_equal_host_series(lib):
    from sim_juncs_gb300.configs import junction_instance
    from sim_juncs_gb300.fields import Fields
    insts = [junction_instance(n=48, res=15.0, phase=p, amplitude=a) for p, a in ((0.3, 1.0), (2.2, 4.0))]
    f = Fields(insts, "f64")
    f.step(2000)
    dev = monitor_phases(f, LOWPASS_INC)
    for q, inst in enumerate(insts):
        mon = f.monitors(q)
        t = np.arange(mon.shape[1]) * (inst.grid.dt * inst.save_span)
        host = extract_phases(t, mon, LOWPASS_INC)
        assert len(dev[q]) == mon.shape[0]
        for a, b in zip(dev[q], host):
            assert a == b
        assert any(d["status"] == _abi.PHASE_OK for d in dev[q])


def test_sweep_sized_batch_equals_series_one_at_a_time(lib, golden):
    # 384 series (the sweep's 96 instances x 4 gap points) in one launch
    s = [x for x in golden if x["kind"] == "junction64"]
    t = np.asarray(s[0]["t"])
    v = np.asarray([x["v"] for x in s] * 48)
    allr = extract_phases(t, v, LOWPASS_INC)
    assert len(allr) == 384
    for q in range(8):
        one = extract_phases(t, v[q:q + 1], LOWPASS_INC)[0]
        assert allr[q] == one and allr[q + 8 * 47] == one
