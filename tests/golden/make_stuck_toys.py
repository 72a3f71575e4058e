"""Writes tests/golden/toys_pwave_stuck.json (+ _events.f64): K*mumu P-wave
toy datasets (Poisson(2000) events at truths jittered by +-10%, generated by
the oracle's restatement of the reference generator) on which the
reference's fitter (MIGRAD + HESSE via oracle/refkit fitfile, started at the
truth) returns the start point unmoved while the gradient there is far from
zero. Test infrastructure: needs oracle/_ref/<arch>/refkit (built from the
reference sources by `make -C oracle ref`)."""
import json
import platform
import struct
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))
from oracle import mforacle as O  # noqa: E402


def main(ntry=120, keep=3):
    spec = json.loads((ROOT / "morefit_gb300" / "specs" / "pwave.json").read_text())
    base = np.array(spec["truth"])
    rng = np.random.default_rng(20261203)
    sets = []
    for t in range(ntry):
        truth = base * (1.0 + rng.uniform(-0.1, 0.1, base.size))
        n = int(np.clip(rng.poisson(2000), 200, 50000))
        sets.append((truth, O.generate("pwave", n, truth=truth, seed=1000 + t)))
    with tempfile.TemporaryDirectory() as td:
        inp, out = Path(td) / "sets.bin", Path(td) / "fits.json"
        with open(inp, "wb") as f:
            for truth, ev in sets:
                f.write(struct.pack("<I", ev.shape[1]))
                f.write(truth.astype(np.float64).tobytes())
                f.write(np.ascontiguousarray(ev, dtype=np.float64).tobytes())
        subprocess.run([str(ROOT / "oracle" / "_ref" / platform.machine() / "refkit"), "fitfile", "pwave", str(inp), str(out)], check=True)
        res = json.loads(out.read_text())
    stuck = [i for i, v in enumerate(res["values"]) if np.array_equal(np.array(v), sets[i][0])][:keep]
    events = np.concatenate([sets[i][1] for i in stuck], axis=1)
    events.astype(np.float64).tofile(HERE / "toys_pwave_stuck_events.f64")
    doc = {"what": "datasets on which the reference's MIGRAD returns the start point", "tried": ntry,
           "stuck_of_tried": sum(np.array_equal(np.array(v), sets[i][0]) for i, v in enumerate(res["values"])),
           "counts": [int(sets[i][1].shape[1]) for i in stuck], "truths": [sets[i][0].tolist() for i in stuck],
           "ref_values": [res["values"][i] for i in stuck], "ref_errors": [res["errors"][i] for i in stuck]}
    (HERE / "toys_pwave_stuck.json").write_text(json.dumps(doc) + "\n")
    print(f"{doc['stuck_of_tried']} of {ntry} reference fits returned the start point; kept {len(stuck)}")


if __name__ == "__main__":
    main()
