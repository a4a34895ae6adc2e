"""Times the reference's own CUDA reconstruction (DQ and UQ kernels compiled
for sm_103a, run by oracle/refrun.py) next to this library on the same
inputs, on one GB300: the 4096^2 configuration-1 images at 4-connectivity
and the 16384^2 spiral at 4-connectivity (the only form the reference
accepts: uint8, square, side a multiple of 512).  Test infrastructure: the
reference cubins under oracle/_ref must have been built from the reference
sources.

    python tests/golden/compare_reference_speed.py [out.json]

Reference time: the span its main() times around MorphologicalReconstruction
(queue allocation to queue free, refrun_harness.cpp), median of 3 process
runs.  Library time: the synchronous iwpp_reconstruct call around the same
span (host clock, median of 5) on device buffers; outputs must match.
"""
import hashlib
import json
import os
import statistics
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
for p in (os.path.join(REPO, "iwpp-mp_gb300"), REPO, HERE):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

import oracle  # noqa: E402
from oracle import refrun  # noqa: E402
import recipes  # noqa: E402
from iwpp import synth  # noqa: E402


def cases():
    for name in ("cfg1_h10", "cfg1_h40", "cfg1_h100"):
        yield name, recipes.RECIPES[name]()
    marker, mask, _ = synth.config2(synth.U8)
    yield "spiral_16384_4conn", (marker, mask)


def main(out_path):
    import torch

    import iwpp

    refrun.build_harness()
    h = iwpp.Handle(0)
    rows = []
    for name, (marker, mask) in cases():
        clipped = np.minimum(marker, mask)
        entry = {"case": name, "size": int(mask.shape[0]), "reference_ms": {}, "library_ms": {}}
        ref_out = None
        for variant in ("dq", "uq"):
            ts = []
            for _ in range(3):
                out, info = refrun.run(variant, marker, mask, timeout=900)
                ts.append(info["ms"])
            entry["reference_ms"][variant] = statistics.median(ts)
            entry.setdefault("reference_rounds", {})[variant] = info["rounds"]
            ref_out = out
        k = torch.from_numpy(mask).cuda()
        m0 = torch.from_numpy(clipped).cuda()
        for variant in ("mutex", "double", "unique", "async"):
            ts = []
            for _ in range(5):
                m = m0.clone()
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                iwpp.reconstruct(m, k, connectivity=4, variant=variant, handle=h)
                ts.append((time.perf_counter() - t0) * 1e3)
            entry["library_ms"][variant] = statistics.median(ts)
            same = bool(np.array_equal(m.cpu().numpy(), ref_out))
            entry.setdefault("same_bytes", {})[variant] = same
        best_ref = min(entry["reference_ms"].values())
        entry["speedup_async_vs_best_reference"] = best_ref / entry["library_ms"]["async"]
        print(json.dumps(entry), flush=True)
        rows.append(entry)
        del k, m0
        torch.cuda.empty_cache()
    with open(out_path, "w") as f:
        json.dump({"generator": "tests/golden/compare_reference_speed.py", "cases": rows}, f, indent=1)
    print("| case | reference DQ ms | reference UQ ms | mutex | double | unique | async | async speed-up | same bytes |")
    print("|---|---|---|---|---|---|---|---|---|")
    for e in rows:
        lm = e["library_ms"]
        print(f"| {e['case']} | {e['reference_ms']['dq']:.2f} | {e['reference_ms']['uq']:.2f} | {lm['mutex']:.2f} | "
              f"{lm['double']:.2f} | {lm['unique']:.2f} | {lm['async']:.2f} | "
              f"{e['speedup_async_vs_best_reference']:.1f}x | {all(e['same_bytes'].values())} |")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "reference_speed.json")
