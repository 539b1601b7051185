"""Generate the nstream and transpose golden fixtures from the reference itself (run where the
reference sources exist).

    make -C oracle ref REF=<ParRes/Kernels checkout>
    python tests/golden/make_neighbours_golden.py

Writes tests/golden/neighbours_golden.json. Each case runs the reference's own driver,
Cxx11/nstream.cc or Cxx11/transpose.cc compiled unmodified with the reference's flags inside
oracle/ref_dump_neighbours.cc, which keeps the driver's arrays after its last iteration. It records
the driver's verdict line and the SHA-256 of every final array (nstream: A, B, C; transpose: A, B),
with a few sampled values. The driver's own initial data are the ones it always uses (nstream:
A = 0, B = C = 2, scalar 3; transpose: A = 0 .. order^2-1 row-major, B = 0).
"""
from __future__ import annotations

import hashlib
import json
import os
import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
REF = ROOT / "oracle" / "_ref"
OUT = Path(__file__).resolve().parent / "neighbours_golden.json"

NSTREAM = [(1, 1), (5, 1003), (10, 4096), (3, 65537)]  # (iterations, length); the driver needs iterations >= 1
TRANSPOSE = [(1, 1, 1), (5, 37, 16), (10, 64, 32), (3, 100, 200), (4, 129, 32)]  # (iterations, order, tile)


def run(binary: str, args: list[str]) -> tuple[list[np.ndarray], str]:
    with tempfile.TemporaryDirectory() as td:
        path = os.path.join(td, "dump.bin")
        res = subprocess.run([str(REF / binary), *args, path], capture_output=True, text=True, check=True)
        data = Path(path).read_bytes()
    arrays, off = [], 0
    while off < len(data):
        (nbytes,) = struct.unpack_from("<Q", data, off)
        off += 8
        arrays.append(np.frombuffer(data[off:off + nbytes], dtype="<f8").copy())
        off += nbytes
    verdict = [ln for ln in res.stdout.splitlines() if "validates" in ln or "ERROR" in ln]
    return arrays, verdict[0] if verdict else ""


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(a.astype("<f8").tobytes()).hexdigest()


def main() -> None:
    nst, tra = [], []
    for it, length in NSTREAM:
        (A, B, C), verdict = run("ref_nstream_dump", [str(it), str(length)])
        nst.append({"iterations": it, "length": length, "verdict": verdict, "A_sha256": sha(A), "B_sha256": sha(B),
                    "C_sha256": sha(C), "A_first_last_hex": [float(A[0]).hex(), float(A[-1]).hex()]})
    for it, order, tile in TRANSPOSE:
        (A, B), verdict = run("ref_transpose_dump", [str(it), str(order), str(tile)])
        tra.append({"iterations": it, "order": order, "tile": tile, "verdict": verdict, "A_sha256": sha(A),
                    "B_sha256": sha(B), "B_first_last_hex": [float(B[0]).hex(), float(B[-1]).hex()]})
    OUT.write_text(json.dumps({
        "generator": "tests/golden/make_neighbours_golden.py",
        "reference": "ParRes/Kernels Cxx11/nstream.cc and Cxx11/transpose.cc via oracle/ref_dump_neighbours.cc",
        "nstream": nst, "transpose": tra}, indent=1) + "\n")
    print(f"wrote {OUT} ({len(nst)} nstream, {len(tra)} transpose cases)")


if __name__ == "__main__":
    main()
