"""Generate eps_reference.json: the reference's own dielectric function
(scripts/utils.py:18-50, class `dielectric_func`, method `get_eps`) for the
susceptibility tuples the stepper consumes.

Run where the reference checkout exists (argument: its root):

    python tests/golden/make_eps_golden.py <reference root>

utils.py is imported unmodified.  It imports h5py and matplotlib for file
input and plotting only; neither is installed here, so stand-in modules take
their place (matplotlib's stand-in accepts the module's `matplotlib.use`
call).  get_eps takes the angular frequency omega = 2 pi f (f in meep units,
1/um with um_scale = 1).

Cases: the Au of the workloads (eps_inf 1, Drude omega_0 = 1, gamma = 0.043,
sigma = 7.3^2; Lorentz 0.33, 0.29, 1.1), their quartz (eps_inf 2.1, Lorentz
10, 0, 0.25), and the reference's own Au and SiO2 entries of
junctions/Au_SiO2_box/junc.geom:60,68, each over f in [0.5, 1.5] x fcen
(fcen = 1/0.7) at 41 points.
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
OUT = os.path.join(HERE, "eps_reference.json")
FCEN = 1 / 0.7

# (name, eps_inf, [(omega_0, gamma, sigma, "drude"|"lorentz")])
CASES = [
    ("workload_au", 1.0, [(1.0, 0.043, 7.3 ** 2, "drude"), (0.33, 0.29, 1.1, "lorentz")]),
    ("workload_quartz", 2.1, [(10.0, 0.0, 0.25, "lorentz")]),
    ("reference_au", 1.0, [(1e-10, 0.04274738474121455, 4.0314052191361974e21, "drude"),
                           (0.3347200880680007, 0.19437961740816426, 11.3629356945, "lorentz")]),
    ("reference_sio2", 1.0, [(9.67865314895427, 0.08065544290795199, 1.12, "lorentz")]),
]


def load_utils(ref_root):
    mpl = types.ModuleType("matplotlib")
    mpl.use = lambda *a, **k: None
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", types.ModuleType("matplotlib.pyplot"))
    sys.modules.setdefault("h5py", types.ModuleType("h5py"))
    spec = importlib.util.spec_from_file_location("ref_utils", os.path.join(ref_root, "scripts", "utils.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def suscept_string(poles):
    return ", ".join(f"({w!r}, {g!r}, {s!r}, {kind})" for w, g, s, kind in poles)


def main(ref_root):
    ut = load_utils(ref_root)
    freqs = np.linspace(0.5, 1.5, 41) * FCEN
    out = {"generator": "tests/golden/make_eps_golden.py", "fcen": FCEN, "freqs": freqs.tolist(), "cases": []}
    for name, eps_inf, poles in CASES:
        with contextlib.redirect_stdout(io.StringIO()):
            d = ut.dielectric_func(suscept_string(poles), eps_inf)
        eps = [complex(d.get_eps(2 * math.pi * f)) for f in freqs]
        out["cases"].append({"name": name, "eps_inf": eps_inf,
                             "poles": [[w, g, s, kind == "drude"] for w, g, s, kind in poles],
                             "eps_re": [e.real for e in eps], "eps_im": [e.imag for e in eps]})
    with open(OUT, "w") as fh:
        json.dump(out, fh, indent=1)
    for c in out["cases"]:
        print(c["name"], c["eps_re"][20], c["eps_im"][20])


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SJ_REFERENCE")
    if not root:
        sys.exit(f"usage: python {sys.argv[0]} <reference checkout root>  (or set SJ_REFERENCE)")
    main(root)
