#!/usr/bin/env python3
"""Writes tests/golden/reference_outputs.json and reference_pulses.json from the reference itself.

Runs the compiled reference (oracle/build_ref.py -> oracle/_ref/bin) on the seeded
inputs of tests/helpers.variant_inputs and records, per case: the sha256 of the input
arrays (pins the input generator), the sha256 of the reference's output fields, their
sums and sums of squares, and the reference's energy.  tests/test_golden.py checks the
oracle against these records on machines without the reference checkout.

Usage (where the reference has been compiled): python tests/golden/make_golden.py
"""
import hashlib
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "tests"))
sys.path.insert(0, str(ROOT / "oracle"))
import conftest  # noqa: E402,F401  (package import path)
import ref_variants  # noqa: E402
import refio  # noqa: E402
from helpers import PULSE_CASES, pulse_inputs, variant_inputs  # noqa: E402

CASES = [(n, s) for n, v in ref_variants.VARIANTS.items()
         if v["kind"] in ("wb_fn", "we_fn") and not v.get("dropin") for s in (4, 30)]


def digest(*arrays):
    h = hashlib.sha256()
    for a in arrays:
        if a is None:
            continue
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def main():
    out = {}
    for name, nsteps in CASES:
        p, f, xy, nbc = variant_inputs(name, seed=100 + nsteps)
        ref = refio.run(name, p.nx, p.ny, refio.STEP, nsteps, fields=f, xy=xy, nbc=nbc)
        rec = {
            "variant": name, "nsteps": nsteps, "seed": 100 + nsteps,
            "input_sha256": digest(f["phi"], f["psi"], f["tmp"], f["tcc"], f["tc"], f["tgamma"], xy, nbc),
            "output_sha256": {k: digest(ref[k]) for k in ("phi", "psi", "tmp")},
            "sum": {k: float(np.sum(ref[k])) for k in ("phi", "psi", "tmp")},
            "sumsq": {k: float(np.sum(ref[k] ** 2)) for k in ("phi", "psi", "tmp")},
            "max_abs": {k: float(np.max(np.abs(ref[k]))) for k in ("phi", "psi", "tmp")},
            "energy": ref["energy"].hex(),
        }
        out[f"{name}/{nsteps}"] = rec
    (HERE / "reference_outputs.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{len(out)} cases")
    # add_circular_wave (wave_common.c:337-351) of the full builds on seeded fields
    pulses = {}
    for name, factor, x, y in PULSE_CASES:
        p, m, phi, psi, xy = pulse_inputs(name)
        ref = refio.run(name, p.nx, p.ny, refio.PULSE, fields={"phi": phi, "psi": psi}, xy=xy, pulse=(factor, x, y))
        pulses[name] = {
            "variant": name, "factor": factor, "x": x, "y": y,
            "input_sha256": digest(phi, psi, xy),
            "output_sha256": digest(ref["phi"]),
            "sum": float(np.sum(ref["phi"])), "sumsq": float(np.sum(ref["phi"] ** 2)),
            "max_abs": float(np.max(np.abs(ref["phi"]))),
        }
    (HERE / "reference_pulses.json").write_text(json.dumps(pulses, indent=1, sort_keys=True) + "\n")
    print(f"{len(pulses)} pulse cases")


if __name__ == "__main__":
    main()
