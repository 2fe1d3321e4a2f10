"""The seeded generators still produce the inputs the reference was run on
for tests/golden/ref_configs.json (SHA-256 of the FP64 points), so the
config-scale digests stay meaningful; the GPU tests repeat the check on
their own platform."""
import json
import os

import numpy as np
import pytest

from dendro_gb300 import datagen
from tests.golden import cases as gcases

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _ref():
    return json.load(open(os.path.join(GOLDEN, "ref_configs.json")))


def test_plain1m_points_reproduced():
    ref = _ref()["plain1m"]
    pts = datagen.workload("gauss1m")
    assert len(pts) == ref["n_pts"]
    assert gcases.sha256_records(pts) == ref["sha_pts"]


def test_batch256_sizes_and_first_clouds_reproduced():
    ref = _ref()
    if "batch256" not in ref:
        pytest.skip("batch256 not generated")
    clouds = ref["batch256"]["clouds"]
    sizes = datagen.cloud_sizes(256, 1e4, 4e6, seed=2)
    assert [c["n_pts"] for c in clouds] == sizes.tolist()
    rng = np.random.Generator(np.random.PCG64(2))
    for i in range(4):
        assert gcases.sha256_records(datagen.mixture(int(sizes[i]), rng)) == clouds[i]["sha_pts"]


def test_portable_exp_is_exact_enough_and_deterministic():
    x = np.linspace(-40.0, 40.0, 200_001)
    e = datagen._exp(x)
    assert np.max(np.abs(e / np.exp(x) - 1.0)) < 5e-16
    # values fixed by the algorithm itself (independent of the platform's libm)
    assert datagen._exp(np.array([0.0]))[0] == 1.0
    got = [v.hex() for v in datagen._exp(np.array([1.0, -2.5, 7.25, 0.3]))]
    assert got == ['0x1.5bf0a8b14576ap+1', '0x1.50385c094f425p-4', '0x1.6006b5d53e8d9p+10', '0x1.599058c8c1a96p+0']
    assert abs(datagen._ln(4e6) - np.log(4e6)) < 1e-15 * 16
