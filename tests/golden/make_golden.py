"""Generate the golden fixtures from the reference itself (run where the reference sources exist).

    make -C oracle ref          # builds oracle/_ref/ from the ParRes/Kernels sources
    python tests/golden/make_golden.py

Writes tests/golden/stencil_golden.json and tests/golden/tiny_out.npz. For every case it runs:
  - oracle/_ref/ref_dump_strict: the reference's own operator (Cxx11/stencil_seq.hpp, included
    unmodified) in the serial driver's loop (Cxx11/stencil.cc:168-191), compiled with strict
    rounding. Its `out` array is recorded as a SHA-256, the norm, and a set of sampled points;
  - oracle/_ref/ref_dump_fast: the same with the reference's -O3 -ffast-math flags, recording the
    largest absolute difference to the strict build (how far the reference's own build drifts);
  - oracle/_ref/stencil and oracle/_ref/stencil-openmp: the reference drivers, recording their
    "Solution validates" verdict and printed L1 norm.
Cases: the reference CI matrix (ci/build-run-prk.sh:334,340-345,372-380: `10 1000` and
`10 200 20 {star,grid} {1..5}`) plus tiny and odd sizes whose whole `out` arrays are stored.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref"
OUT_JSON = Path(__file__).resolve().parent / "stencil_golden.json"
OUT_NPZ = Path(__file__).resolve().parent / "tiny_out.npz"

CI_CASES = [("star", 2, 1000, 10, 32)] + [(p, r, 200, 10, 20) for p in ("star", "grid") for r in range(1, 6)]
TINY_CASES = [(p, r, n, 3, 4) for p in ("star", "grid") for r in range(1, 6) for n in (2 * r + 1, 2 * r + 2, 16, 37)]


def dump(kind: str, case) -> tuple[np.ndarray, float]:
    pattern, r, n, it, tile = case
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "out.bin")
        res = subprocess.run([str(REF / f"ref_dump_{kind}"), str(it), str(n), str(tile), pattern, str(r), path],
                             check=True, capture_output=True, text=True)
        out = np.fromfile(path, dtype="<f8").reshape(n, n)
    norm = float.fromhex(res.stdout.split()[1])
    return out, norm


def driver(binary: str, case) -> dict:
    pattern, r, n, it, tile = case
    env = dict(os.environ, OMP_NUM_THREADS="2")
    res = subprocess.run([str(REF / binary), str(it), str(n), str(tile), pattern, str(r)], capture_output=True,
                         text=True, env=env)
    norm_line = [ln for ln in res.stdout.splitlines() if ln.startswith("L1 norm")]
    return {"rc": res.returncode, "validates": "Solution validates" in res.stdout,
            "l1_norm_line": norm_line[0] if norm_line else None}


def samples(n: int, r: int, rng: np.random.Generator) -> list[tuple[int, int]]:
    lo, hi = r, n - r - 1
    pts = {(lo, lo), (lo, hi), (hi, lo), (hi, hi), ((lo + hi) // 2, (lo + hi) // 2)}
    while len(pts) < 32:
        pts.add((int(rng.integers(lo, hi + 1)), int(rng.integers(lo, hi + 1))))
    return sorted(pts)


def main() -> None:
    rng = np.random.default_rng(20260101)
    cases = []
    for case in CI_CASES:
        pattern, r, n, it, tile = case
        strict, norm = dump("strict", case)
        fast, _ = dump("fast", case)
        pts = samples(n, r, rng)
        cases.append({
            "pattern": pattern, "radius": r, "n": n, "iterations": it, "tile": tile,
            "norm_hex": norm.hex(),
            "out_sha256": hashlib.sha256(strict.astype("<f8").tobytes()).hexdigest(),
            "points": [[i, j, float(strict[i, j]).hex()] for i, j in pts],
            "fastmath_max_abs_diff": float(np.abs(fast - strict).max()),
            "ref_stencil": driver("stencil", case),
            "ref_stencil_openmp": driver("stencil-openmp", case),
        })
    tiny = {}
    for case in TINY_CASES:
        pattern, r, n, it, tile = case
        strict, norm = dump("strict", case)
        tiny[f"{pattern}{r}_n{n}_k{it}"] = strict
    OUT_JSON.write_text(json.dumps({
        "generator": "tests/golden/make_golden.py",
        "reference": "ParRes/Kernels Cxx11 stencil (stencil_seq.hpp via oracle/ref_dump.cc)",
        "cases": cases,
        "tiny": [{"key": f"{p}{r}_n{n}_k{it}", "pattern": p, "radius": r, "n": n, "iterations": it, "tile": t}
                 for p, r, n, it, t in TINY_CASES],
    }, indent=1) + "\n")
    np.savez_compressed(OUT_NPZ, **tiny)
    print(f"wrote {OUT_JSON} ({len(cases)} cases) and {OUT_NPZ} ({len(tiny)} arrays)")


if __name__ == "__main__":
    main()
