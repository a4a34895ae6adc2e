"""The oracle pinned to the reference itself.

tests/golden/reference_outputs.json holds, for each input recipe in
tests/golden/recipes.py, the SHA-256 of the output of the reference's own
CUDA reconstruction (IWPP MP DQ and IWPP MP UQ kernels, compiled unmodified
for sm_103a and run on a GB300 by tests/golden/make_reference_fixtures.py).
The recipes regenerate bit-identical inputs on any host, so the CPU oracle
(and, on a GPU, libiwpp) must reproduce those hashes exactly.
"""
import hashlib
import json
import os
import sys

import numpy as np
import pytest

import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import recipes  # noqa: E402

FIXTURES = json.load(open(os.path.join(HERE, "golden", "reference_outputs.json")))["cases"]
SMALL = [c for c in FIXTURES if c["size"] <= 2048]
LARGE = [c for c in FIXTURES if c["size"] > 2048]


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def test_fixture_file_covers_every_recipe_and_both_variants_agree():
    assert {c["recipe"] for c in FIXTURES} == set(recipes.RECIPES)
    for c in FIXTURES:
        assert c["reference"]["dq"]["sha256"] == c["reference"]["uq"]["sha256"], c["recipe"]


@pytest.mark.parametrize("case", SMALL + LARGE, ids=lambda c: c["recipe"])
def test_oracle_reproduces_reference_output(case):
    marker, mask = recipes.RECIPES[case["recipe"]]()
    out = oracle.reconstruct(oracle.clip(marker, mask), mask, 4)
    assert _sha(out) == case["reference"]["dq"]["sha256"]


@pytest.mark.gpu
@pytest.mark.parametrize("variant", ["mutex", "double", "unique", "async"])
def test_library_reproduces_reference_output(variant):
    import iwpp
    import torch
    for case in FIXTURES:
        marker, mask = recipes.RECIPES[case["recipe"]]()
        m = torch.from_numpy(marker).cuda()
        k = torch.from_numpy(mask).cuda()
        iwpp.clip(m, k)
        iwpp.reconstruct(m, k, connectivity=4, variant=variant)
        assert _sha(m.cpu().numpy()) == case["reference"]["dq"]["sha256"], (variant, case["recipe"])
