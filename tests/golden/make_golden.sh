#!/usr/bin/env bash
# Regenerates the golden vectors under tests/golden/ from the reference's own
# generator, fitter and Minuit2 (oracle/refkit, built from the reference
# sources by `make -C oracle ref`). Needs the reference sources
# (MOREFIT_REFERENCE=<reference tree>, or a copy staged by `make -C oracle
# stage`); the GPU host only reads the committed outputs.
set -euo pipefail
HERE="$(cd "$(dirname "$0")" && pwd)"
ROOT="$(cd "$HERE/../.." && pwd)"
make -C "$ROOT/oracle" ref -j"$(nproc)" >/dev/null
K="$ROOT/oracle/_ref/$(uname -m)/refkit"
"$K" golden pwave 1000 "$HERE/pwave_n1000.json" "$HERE/pwave_n1000_events.f64"
"$K" golden mass 1000 "$HERE/mass_n1000.json" "$HERE/mass_n1000_events.f64"
"$K" golden mass 100000 "$HERE/mass_n100000.json"
"$K" golden mass_w 1000 "$HERE/mass_w_n1000.json" "$HERE/mass_w_n1000_events.f64"
"$K" golden mass_w 100000 "$HERE/mass_w_n100000.json"
"$K" golden cbpoly 1000 "$HERE/cbpoly_n1000.json" "$HERE/cbpoly_n1000_events.f64"
"$K" golden cbpoly 100000 "$HERE/cbpoly_n100000.json"
"$K" golden pwave 1000000 "$HERE/pwave_n1000000.json"
"$K" golden spwave 2000 "$HERE/spwave_n2000.json" "$HERE/spwave_n2000_events.f64"
"$K" golden spwave 20000 "$HERE/spwave_n20000.json"
"$K" toys pwave 1000 2000 0.1 "$HERE/toys_pwave_ref.json"
python3 "$HERE/make_stuck_toys.py"
# the reference's plotter (matplotlib and ROOT text, per-bin integrals)
T="$(mktemp -d)"
for wv in mass:m mass_w:m cbpoly:x pwave:ctl pwave:ctk pwave:phi; do
  w="${wv%%:*}"; v="${wv##*:}"
  "$K" plot "$w" 100000 "$v" 100 "$T/plot_${w}_${v}.py" "$HERE/plot_${w}_${v}.json"
done
rm -r "$T"
python3 "$HERE/extract_specs.py"
