"""Extract the reference's own known-answer values into reference_goldens.json.

Reads rebop's test sources as text (the Rust crate cannot be built here) and
records each golden with the file:line it came from:
  * src/gillespie.rs  rate_lma (check_rate cases), jump_affect,
                      rate_conversion / rate_sparse, jump_conversion
  * src/expr.rs       test_eval / test_eval_max
  * tests/test_rebop.py test_fixed_seed (final S, I, R at rng=42)
plus the numpy seed the reference's Python wrapper derives for rng=42
(python/rebop/gillespie.py:139-140), computed with numpy itself.

Usage: python tests/golden/extract_reference_goldens.py REFERENCE_ROOT
(or set REBOP_REFERENCE to the rebop source tree).
"""

from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent


def _nums(s: str) -> list:
    return [int(x) for x in re.findall(r"-?\d+", s)]


def extract(ref: Path) -> dict:
    out: dict = {"source": "rebop v0.9.7", "rate_lma": [], "jump_affect": [], "rate_sparse": [],
                 "expr_eval": [], "fixed_seed": {}}
    g = (ref / "src/gillespie.rs").read_text().splitlines()
    species = None
    for i, line in enumerate(g, 1):
        m = re.search(r"let species = \[([^\]]*)\];", line)
        if m:
            species = _nums(m.group(1))
        m = re.search(r"check_rate\(&Rate::lma\(([-\d.eE]+), \[([^\]]*)\]\), &species, ([-\d.eE]+)\);", line)
        if m and species is not None:
            out["rate_lma"].append({"rate": float(m.group(1)), "exponents": _nums(m.group(2)),
                                    "species": species, "expected": float(m.group(3)),
                                    "where": f"src/gillespie.rs:{i}"})
        m = re.search(r"let rate = Rate::lma\(([-\d.eE]+), \[([^\]]*)\]\);", line)
        if m and i + 1 <= len(g):
            nxt = g[i]  # the following line
            m2 = re.search(r"rate\.sparse\(\), Rate::LMASparse\(([-\d.eE]+), vec!\[(.*)\]\)\);", nxt)
            if m2:
                pairs = [tuple(int(v) for v in p) for p in re.findall(r"\((\d+), (\d+)\)", m2.group(2))]
                out["rate_sparse"].append({"rate": float(m.group(1)), "dense": _nums(m.group(2)),
                                           "sparse": pairs, "where": f"src/gillespie.rs:{i + 1}"})
    # jump_affect: Jump::new([...]) applied to vec![10; 4] -> expected
    text = "\n".join(g)
    m = re.search(r"fn jump_affect\(\) \{(.*?)\n    \}", text, re.S)
    if m:
        body = m.group(1)
        start = text[:m.start()].count("\n") + 1
        dj = re.search(r"Jump::new\(\[([^\]]*)\]\)", body)
        init = re.search(r"vec!\[(-?\d+); (\d+)\]", body)
        exp = re.search(r"assert_eq!\(species, vec!\[([^\]]*)\]\)", body)
        out["jump_affect"].append({"differences": _nums(dj.group(1)),
                                   "species": [int(init.group(1))] * int(init.group(2)),
                                   "expected": _nums(exp.group(1)), "where": f"src/gillespie.rs:{start}"})
    e = (ref / "src/expr.rs").read_text().splitlines()
    for i, line in enumerate(e, 1):
        m = re.search(r'let pe: PExpr = "([^"]*)"\.parse\(\)\.unwrap\(\);', line)
        if not m:
            continue
        expr = m.group(1)
        names, species_vals, expected = {}, None, None
        for j in range(i, min(i + 20, len(e))):
            mm = re.search(r'init\.insert\("(\w+)"\.to_string\(\), (\d+)\);', e[j])
            if mm:
                names[mm.group(1)] = int(mm.group(2))
            mm = re.search(r"let species = vec!\[([^\]]*)\];", e[j])
            if mm:
                species_vals = _nums(mm.group(1))
            mm = re.search(r"\.eval\(&species\),?\s*$", e[j])
            mm2 = re.search(r"\.eval\(&species\), ([-\d.eE]+)\);", e[j])
            if mm2:
                expected = float(mm2.group(1))
                break
            if mm:
                val = re.search(r"^\s*([-\d.eE]+)\s*$", e[j + 1])
                if val:
                    expected = float(val.group(1))
                break
            if j > i and "let pe: PExpr" in e[j]:
                break
        if expected is not None and species_vals is not None:
            out["expr_eval"].append({"expr": expr, "species_index": names, "species": species_vals,
                                     "expected": expected, "where": f"src/expr.rs:{i}"})
    t = (ref / "tests/test_rebop.py").read_text().splitlines()
    for i, line in enumerate(t, 1):
        if "def test_fixed_seed" in line:
            block = t[i:i + 8]
            run = next(b for b in block if "sir.run(" in b)
            seed = int(re.search(r"rng=(\d+)", run).group(1))
            vals = {}
            for b in block:
                mm = re.search(r"assert ds\.(\w+)\[-1\] == (\d+)", b)
                if mm:
                    vals[mm.group(1)] = int(mm.group(2))
            init = {k: int(v) for k, v in re.findall(r'"(\w+)": (\d+)', run)}
            out["fixed_seed"] = {"rng": seed, "final": vals, "init": init,
                                 "tmax": float(re.search(r"tmax=(\d+)", run).group(1)),
                                 "nb_steps": int(re.search(r"nb_steps=(\d+)", run).group(1)),
                                 "numpy_seed": int(np.random.default_rng(seed).integers(
                                     np.iinfo(np.uint64).max, dtype=np.uint64)),
                                 "where": f"tests/test_rebop.py:{i}"}
    out["vilar"] = extract_vilar(ref)
    return out


def extract_vilar(ref: Path) -> dict:
    """Parameters, reactions and run arguments of the Vilar oscillator benchmark
    as the run-time API builds it (benchmarks/benches/vilar/vilar.py)."""
    path = "benchmarks/benches/vilar/vilar.py"
    lines = (ref / path).read_text().splitlines()
    params, reactions, run = {}, [], None
    for i, line in enumerate(lines, 1):
        m = re.match(r"^(\w+) = ([-\d.eE]+)\s*$", line)
        if m:
            params[m.group(1)] = float(m.group(2))
            continue
        m = re.search(r"\.add_reaction\((\w+), \[([^\]]*)\], \[([^\]]*)\]\)", line)
        if m:
            reactions.append({"rate_param": m.group(1), "rate": params[m.group(1)],
                              "reactants": re.findall(r'"(\w+)"', m.group(2)),
                              "products": re.findall(r'"(\w+)"', m.group(3)),
                              "where": f"{path}:{i}"})
            continue
        m = re.search(r"for _ in range\((\d+)\):", line)
        if m:
            n_traj = int(m.group(1))
        m = re.search(r"\.run\(\{([^}]*)\}, tmax=([-\d.eE]+), nb_steps=(\d+)\)", line)
        if m:
            run = {"init": {k: int(v) for k, v in re.findall(r'"(\w+)": (\d+)', m.group(1))},
                   "tmax": float(m.group(2)), "nb_steps": int(m.group(3)),
                   "n_traj": n_traj, "where": f"{path}:{i}"}
    return {"params": params, "reactions": reactions, "run": run}


if __name__ == "__main__":
    # the reference source tree: first argument, else $REBOP_REFERENCE
    arg = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("REBOP_REFERENCE")
    if not arg:
        sys.exit("usage: extract_reference_goldens.py <rebop source tree>  (or set REBOP_REFERENCE)")
    ref = Path(arg)
    data = extract(ref)
    (HERE / "reference_goldens.json").write_text(json.dumps(data, indent=1) + "\n")
    print({k: (len(v) if isinstance(v, list) else v) for k, v in data.items()})
