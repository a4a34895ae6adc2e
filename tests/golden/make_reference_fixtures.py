"""Generates tests/golden/reference_outputs.json by running the reference's
own CUDA reconstruction (DQ and UQ variants, oracle/refrun.py) on every
recipe in recipes.py.  Needs a GB300 and the reference cubins under
oracle/_ref (built from the reference sources).

    python tests/golden/make_reference_fixtures.py <out.json>

Each entry records the recipe, the SHA-256 of the reference's output per
variant, the reference's round count, and whether the CPU oracle agrees.
"""
import hashlib
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(REPO, "iwpp-mp_gb300"), REPO, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import oracle  # noqa: E402
from oracle import refrun  # noqa: E402
import recipes  # noqa: E402


def sha(a):
    return hashlib.sha256(a.tobytes()).hexdigest()


def main(out_path):
    refrun.build_harness()
    entries = []
    for name, fn in recipes.RECIPES.items():
        marker, mask = fn()
        expect = oracle.reconstruct(oracle.clip(marker, mask), mask, 4)
        entry = {"recipe": name, "size": int(marker.shape[0]), "connectivity": 4,
                 "oracle_sha256": sha(expect), "reference": {}}
        for variant in ("dq", "uq"):
            t0 = time.time()
            out, info = refrun.run(variant, marker, mask)
            entry["reference"][variant] = {"sha256": sha(out), "rounds": info["rounds"],
                                           "restarts": info["restarts"], "seconds": round(time.time() - t0, 3),
                                           "matches_oracle": bool((out == expect).all())}
        print(json.dumps(entry), flush=True)
        entries.append(entry)
    with open(out_path, "w") as f:
        json.dump({"generator": "tests/golden/make_reference_fixtures.py",
                   "reference": "oliveira-mathias/IWPP-MP, IWPP MP DQ and IWPP MP UQ kernels compiled for sm_103a",
                   "cases": entries}, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "reference_outputs.json"))
