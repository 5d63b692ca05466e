"""Extract the golden vectors the oracle is pinned against.

The reference (fluid-sim) is JavaScript and cannot run in this environment, so
the pins are the reference's OWN committed run outputs:

* ``results/validation.json`` -- written by ``validate/run.js`` under Node 24
  (f64 CPU solver): the Taylor-Green study (``validate/studies.js:121-177``),
  the translating-Gaussian advection study (``:48-97``), the dt x N convergence
  table (``:191-230``), the explicit-diffusion amplification sweep and the
  projection-iteration sweep (``:247-454``).
* ``results/gpu-verify.json`` -- written by ``tools/gputest.html`` on the
  reference WebGPU backend (f32): Poisson residual curves for Jacobi,
  red-black and multigrid at 64^2 from the seed-777 random field, the
  GPU-vs-CPU agreement figures and the scheme energies.

Run from the repository root with the reference checked out:

    python tests/golden/extract_golden.py /path/to/fluid-sim

It writes ``tests/golden/reference_results.json`` (committed); the tests read
only that file.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    val = json.loads((ref / "results" / "validation.json").read_text())
    gpu = json.loads((ref / "results" / "gpu-verify.json").read_text())

    tg = val["taylorGreen"]
    out = {
        "source": {
            "validation.json": {"env": val["env"]},
            "gpu-verify.json": {"adapter": gpu["adapter"]},
        },
        "taylorGreen": {
            "n": tg["n"], "nu": tg["nu"], "dt": tg["dt"], "T": tg["T"],
            "schemes": {
                name: {
                    "trace": [{k: p[k] for k in ("t", "relL2", "ke", "enstrophy", "maxDiv", "cgIterations")}
                              for p in sch["trace"]],
                    "nuNumerical": sch["nuNumerical"],
                    "measuredDecayRate": sch["measuredDecayRate"],
                    "decayFitR2": sch["decayFitR2"],
                }
                for name, sch in tg["schemes"].items()
            },
        },
        "advection": {
            k: val["advection"][k] for k in ("n", "dt", "steps", "sigma0")
        } | {
            "schemes": {
                name: {"trace": sch["trace"], "peakInitial": sch["peakInitial"],
                       "numericalDiffusion": sch["numericalDiffusion"]}
                for name, sch in val["advection"]["schemes"].items()
            }
        },
        "convergence": {
            k: val["convergence"][k] for k in ("nu", "T", "scheme", "Ns", "dts")
        } | {"table": [{"n": r["n"], "errors": r["errors"]} for r in val["convergence"]["table"]]},
        "explicitDiffusion": {
            "n": val["stability"]["explicitDiffusion"]["n"],
            "nu": val["stability"]["explicitDiffusion"]["nu"],
            "isolated": [{k: p[k] for k in ("diffusionNumber", "dt", "predictedAmplification",
                                            "measuredAmplification", "amplitudes", "unstable")}
                         for p in val["stability"]["explicitDiffusion"]["isolated"]],
            "measuredBoundary": val["stability"]["explicitDiffusion"]["measuredBoundary"],
        },
        "projectionIterations": val["stability"]["projectionIterations"],
        "gpu": {
            "poissonCurves": gpu["poissonCurves"],
            "advection": gpu["advection"],
            "divergence": gpu["divergence"],
            "projection": gpu["projection"],
            "fullStep": gpu["fullStep"],
            "macCormack": gpu["macCormack"],
            "schemeEnergy": gpu["schemeEnergy"],
            "gpuSolid": gpu["gpuSolid"],
            "gpuSolidAgreement": gpu["gpuSolidAgreement"],
        },
    }
    dst = Path(__file__).resolve().parent / "reference_results.json"
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python extract_golden.py <path of a fluid-sim checkout>")
    main(sys.argv[1])
