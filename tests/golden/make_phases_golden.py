"""Generate phases_reference.json: what the reference's CEP/envelope extraction
(scripts/phases.py, class `signal`, as `opt_pulse_full` calls it at
scripts/phases.py:735-758) returns for a set of monitor series.

Run where the reference checkout exists (argument: its root):

    python tests/golden/make_phases_golden.py <reference root>

phases.py is imported unmodified.  Its module imports h5py and matplotlib
for file input and plotting only; neither is installed here, so empty stand-in
modules take their place (the extraction path uses neither).  NumPy 2 removed
np.trapz, which the extraction calls; it is aliased to np.trapezoid, the same
trapezoidal integral under its current name.

Series: (1) seeded synthetic pulses in the form the CEP/amplitude sweep
records, a Gaussian-envelope carrier sampled every 20 steps with CEP drawn
from [0, 2 pi) and amplitude log-uniform in [0.1, 10]; (2) the Ex and Ez gap
monitors of the 64^3 junction run for 2000 steps on the FP64 oracle.  For each
series the file holds the input and signal's f0, phi (_phi_corr), t0
correction, the envelope peak opt_pulse_full stores as the amplitude, the
envelope's mean, width and skewness (get_skewness), f0's bin, the band of the
phase fit, the low-pass strength reached and t0; or, where the reference
raises (its phase fit needs at least five frequency bins in the band), the
exception's type and message.  "sensitivity" records how far the reference's
own answers move when the input is perturbed by 1e-15 relative: the
synthetic pulses, whose carrier sits near the sampling's Nyquist frequency,
go through four low-pass steps that leave near-zero bins inside the band,
and their phase fit then depends on rounding.
"""
import contextlib
import importlib.util
import io
import json
import math
import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
OUT = os.path.join(HERE, "phases_reference.json")
SEED = 11
N_SYNTH = 12


def load_phases(ref_root):
    for name in ("h5py", "matplotlib", "matplotlib.pyplot"):
        sys.modules.setdefault(name, types.ModuleType(name))
    if not hasattr(np, "trapz"):
        np.trapz = np.trapezoid
    spec = importlib.util.spec_from_file_location("ref_phases", os.path.join(ref_root, "scripts", "phases.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.verbose = 0
    return mod


def synthetic_series(rng):
    """A pulse as the sweep's gap monitors record it: fcen = 1/0.7, a Gaussian
    envelope of width 1/(2 pi fwidth) with fwidth = 0.5, sampled every 20
    steps of dt = 0.5 / 30."""
    dt = 20 * 0.5 / 30.0
    n = 200
    t = np.arange(n) * dt
    fcen, width = 1 / 0.7, 1 / (2 * math.pi * 0.5)
    out = []
    for _ in range(N_SYNTH):
        phase = rng.uniform(0.0, 2 * math.pi)
        amp = math.exp(rng.uniform(math.log(0.1), math.log(10.0)))
        t0 = rng.uniform(10.0, 16.0)
        v = amp * np.exp(-0.5 * ((t - t0) / width) ** 2) * np.cos(2 * math.pi * fcen * (t - t0) + phase)
        v += 1e-3 * amp * rng.standard_normal(n)
        out.append({"kind": "synthetic", "cep": phase, "amplitude": amp, "t0": t0, "fcen": fcen,
                    "t": t.tolist(), "v": v.tolist()})
    return out


def junction_series():
    from oracle.oracle import OracleFields
    from sim_juncs_gb300.configs import junction_instance
    inst = junction_instance()
    o = OracleFields(inst)
    o.step(2000)
    mon = o.monitors()
    o.close()
    t = np.arange(mon.shape[1]) * (inst.grid.dt * inst.save_span)
    return [{"kind": "junction64", "monitor": q, "t": t.tolist(), "v": mon[q].tolist()} for q in range(mon.shape[0])]


def extract(ph, t, v):
    t, v = np.asarray(t), np.asarray(v)
    with contextlib.redirect_stdout(io.StringIO()):
        s = ph.signal(t, v, lowpass_inc=2.0)
        env = s.get_envelope()
        k = int(np.argmax(env))
        mu, sig, skew, _ = s.get_skewness()
        band = s._get_freq_fwhm()
    return {"f0": float(s.f0), "phi": float(s._phi_corr), "t0_corr": float(s._t0_corr),
            "amp": [float(env[k].real), float(env[k].imag)], "mu": float(mu), "sig": float(sig),
            "skew": float(skew), "f0_ind": int(s.f0_ind), "band": [int(band[0]), int(band[1])],
            "lowpass_strength": float(s._low_stren), "t0": float(s.t0)}


SENS_KEYS = ("f0", "phi", "t0_corr", "amp", "mu", "sig", "skew")


def sensitivity(ph, t, v, ref, rng):
    """How far the reference's own answers move when its input moves by
    1e-15 relative (three seeded perturbations): near-zero spectral bins in
    the band make the phase fit depend on rounding, and a port can match such
    a series no closer than this."""
    out = {k: 0.0 for k in SENS_KEYS}
    v = np.asarray(v)
    for _ in range(3):
        try:
            r = extract(ph, t, v * (1 + 1e-15 * rng.standard_normal(v.size)))
        except Exception:
            return {k: float("inf") for k in SENS_KEYS}
        for k in SENS_KEYS:
            out[k] = max(out[k], float(np.max(np.abs(np.asarray(r[k]) - np.asarray(ref[k])))))
    return out


def main(ref_root):
    ph = load_phases(ref_root)
    rng = np.random.default_rng(SEED)
    series = synthetic_series(rng) + junction_series()
    prng = np.random.default_rng(SEED + 1)
    for s in series:
        try:
            s["reference"] = extract(ph, s["t"], s["v"])
        except Exception as e:  # the reference raises on some series; that is recorded too
            s["reference"] = {"error": type(e).__name__, "message": str(e)}
        else:
            s["sensitivity"] = sensitivity(ph, s["t"], s["v"], s["reference"], prng)
    with open(OUT, "w") as fh:
        json.dump({"generator": "tests/golden/make_phases_golden.py", "seed": SEED, "series": series}, fh)
    for s in series:
        r = s["reference"]
        print(s["kind"], s.get("cep", s.get("monitor")), r.get("error") or (r["f0"], r["phi"], r["amp"], r["skew"]))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SJ_REFERENCE")
    if not root:
        sys.exit(f"usage: python {sys.argv[0]} <reference checkout root>  (or set SJ_REFERENCE)")
    main(root)
