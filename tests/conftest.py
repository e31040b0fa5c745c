import gzip
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "saige-gpu_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built libsaigegpu.so")


@pytest.fixture(scope="session")
def golden_plink():
    bed = gzip.open(os.path.join(GOLDEN, "plink_1000x10k.bed.gz")).read()
    ph = np.load(os.path.join(GOLDEN, "pheno_1000.npz"))
    return bed, int(ph["n_fam"]), int(ph["m_bim"]), ph


@pytest.fixture(scope="session")
def gpu_ctx():
    from saigegpu import build, Context
    build.build_lib()
    ctx = Context(0)
    yield ctx
    ctx.close()
