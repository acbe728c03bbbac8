import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libpars_gpu.so")


@pytest.fixture(scope="session")
def port():
    import oracle
    return oracle.port()


@pytest.fixture(scope="session")
def ctx():
    from pars_gb300 import native
    c = native.Context(0)
    yield c
    c.close()


def golden(name):
    return np.load(os.path.join(GOLDEN, name))


def golden_field(data, prefix="field_"):
    from pars_gb300.workloads import Field
    return Field(data[prefix + "xyz"], data[prefix + "offset"], data[prefix + "spacing"], data[prefix + "size"])


def golden_curves(data, prefix):
    out = []
    for b in range(int(data[prefix + "batches"])):
        item = {"vertices": data.get(f"{prefix}{b}_vertices"), "indices": data.get(f"{prefix}{b}_indices"),
                "colors": data.get(f"{prefix}{b}_colors"), "rank": int(data[f"{prefix}{b}_rank"]),
                "round": int(data[f"{prefix}{b}_round"])}
        out.append(item)
    return out


def particles_from(data, key):
    import oracle
    return np.frombuffer(data[key].tobytes(), oracle.PARTICLE_DTYPE).copy()


def assert_colors_equal(actual, expected, ulp_tolerance=0.0):
    """Compares only the colours the reference writes (NaN in `expected` marks
    never-written entries).  ulp_tolerance = 0 means bit-exact."""
    mask = ~np.isnan(expected).any(axis=1)
    a, e = actual[mask], expected[mask]
    if ulp_tolerance == 0:
        assert np.array_equal(a, e, equal_nan=True), f"{np.sum(np.any(a != e, axis=1))} colours differ"
    else:
        both_nan = np.isnan(a) & np.isnan(e)
        diff = np.where(both_nan, 0.0, np.abs(a.astype(np.float64) - e.astype(np.float64)))
        assert np.nanmax(diff) <= ulp_tolerance, f"max colour difference {np.nanmax(diff)}"
