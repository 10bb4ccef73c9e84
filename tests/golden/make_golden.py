"""Generates tests/golden/reference_lsb16.json from the REFERENCE program itself.

The reference's mySort and globalShuffle (mpi/mpi_lsbsort.cpp:493-597,
RADIX 16) are compiled from its own source file by ``make -C oracle ref``
(one-rank MPI shim) and run on inputs from the project's seeded generator
(oracle.generate: splitmix64 keys, value = index, mpi/mpi_lsbsort.cpp:686-692).
For every case the fixture records SHA-256 digests of

* the input (pins the generator),
* the sorted output of mySort,
* globalShuffle(input, d) for each digit d (one pass on the input),
* the state after passes 0..d (mySort's intermediate arrays),

and, for n <= 64, the full output. Digests are over the (n, 2) little-endian
uint64 array, i.e. the raw bytes of the SortElement array.

Run from the repository root:  python tests/golden/make_golden.py
This needs the reference checkout; the fixture it writes does not.
"""
from __future__ import annotations

import hashlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import numpy as np  # noqa: E402

import oracle as O  # noqa: E402

OUT = os.path.join(HERE, "reference_lsb16.json")

CASES = []
for dist in ("uniform", "low32", "zipf", "equal", "nearly_sorted"):
    for n in (0, 1, 2, 3, 17, 100, 4095, 4096, 4097, 65535, 65536, 65537, 300007):
        CASES.append((dist, n, 7))
CASES += [("uniform", 1 << 20, 1), ("zipf", 1 << 20, 3), ("uniform", 1 << 24, 0)]


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<u8").tobytes()).hexdigest()


def main() -> None:
    O.build(with_ref=True)
    if not O.ref_available():
        raise SystemExit("reference build missing")
    cases = []
    for dist, n, seed in CASES:
        a = O.generate(n, O.DIST_NAMES[dist], seed)
        out = O.ref_mysort(a)
        rec = {
            "dist": dist,
            "n": n,
            "seed": seed,
            "digit_bits": 16,
            "input_sha256": digest(a),
            "sorted_sha256": digest(out),
            "pass_sha256": [digest(O.ref_global_shuffle(a, d)) for d in range(4)],
        }
        cur, after = a, []
        for d in range(4):
            cur = O.ref_global_shuffle(cur, d)
            after.append(digest(cur))
        rec["after_pass_sha256"] = after
        if n <= 64:
            rec["sorted"] = [[f"{int(k):016x}", int(v)] for k, v in out]
        cases.append(rec)
        print(dist, n, seed, rec["sorted_sha256"][:16], flush=True)
    doc = {
        "what": "reference mySort/globalShuffle outputs (mpi/mpi_lsbsort.cpp, RADIX 16, 1 rank)",
        "generator": "oracle.generate: key = splitmix64(seed, i) (variants per dist), val = i",
        "cases": cases,
    }
    with open(OUT, "w") as f:
        json.dump(doc, f, indent=1)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
