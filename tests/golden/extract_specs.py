"""Writes morefit_gb300/specs/<workload>.json from the golden files.

A spec is what the reference's fitter hands its compute backend for one
model (include/fitter.hh:321-658): the kernel descriptions (input columns,
parameter names, one get_kernel() string per output) and the hoisted
parameter-buffer expressions the fitter evaluates on the host before each
launch (fitter.hh:1063-1072). The golden values themselves stay in
tests/golden/.
"""
import json
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent.parent / "morefit_gb300" / "specs"

ANGLES = {"ctl": [-1.0, 1.0], "ctk": [-1.0, 1.0], "phi": [-3.141592653589793, 3.141592653589793]}
RANGES = {"mass": {"m": [5000.0, 5600.0]}, "mass_w": {"m": [5000.0, 5600.0], "w": [0.0, 2.0]},
          "cbpoly": {"x": [-1.0, 1.0]}, "pwave": ANGLES, "spwave": ANGLES}


def main():
    OUT.mkdir(parents=True, exist_ok=True)
    for wl, src in (("mass", "mass_n1000.json"), ("mass_w", "mass_w_n1000.json"), ("cbpoly", "cbpoly_n1000.json"),
                    ("pwave", "pwave_n1000.json"), ("spwave", "spwave_n2000.json")):
        g = json.loads((HERE / src).read_text())
        spec = {k: g[k] for k in ("workload", "dimensions", "parameters", "truth", "kernels", "event_buffers",
                                  "lh_buffers", "grad_buffers", "hessian_buffers")}
        for k in ("weight", "fisher_buffers"):
            if k in g:
                spec[k] = g[k]
        # plotter integrals per variable (oracle/refkit plot), parameters symbolic
        for f in sorted(HERE.glob(f"plot_{wl}_*.json")):
            pg = json.loads(f.read_text())
            if pg["workload"] != wl:
                continue
            spec.setdefault("integrals", {})[pg["variable"]] = pg["integral"]
            spec["tex"] = pg["tex"]
        spec["ranges"] = [RANGES[wl][d] for d in g["dimensions"]]
        spec["seed"] = g["seed"]
        (OUT / f"{wl}.json").write_text(json.dumps(spec, indent=1) + "\n")
        print("wrote", OUT / f"{wl}.json", file=sys.stderr)


if __name__ == "__main__":
    main()
