import hashlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); run with -m gpu")


def manifest() -> dict:
    with open(os.path.join(GOLDEN, "manifest.json")) as f:
        return json.load(f)


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def conn_hash(rowptr, cols) -> str:
    return hashlib.sha256(np.ascontiguousarray(rowptr, dtype="<u8").tobytes() +
                          np.ascontiguousarray(cols, dtype="<u4").tobytes()).hexdigest()


def mbs_sha(z: np.ndarray) -> str:
    n, N = z.shape
    h = hashlib.sha256()
    h.update(np.int32(N).tobytes())
    h.update(np.uint64(n).tobytes())
    h.update(np.ascontiguousarray(z, dtype="<u2").tobytes())
    return h.hexdigest()


def synthetic_xml(name: str, tmpdir: str) -> str:
    """Regenerate the seeded synthetic system of a manifest entry."""
    from cosmo_gb300.synthetic import SyntheticSystem, make_system
    s = manifest()[name]["system"]
    sysd = SyntheticSystem(s["space"], s["nv"], s["zv"], s["twom"], s["parity"], s["jj"], s["seed"], name=name)
    return make_system(tmpdir, sysd)[1]


def problem_for(name: str, tmpdir: str):
    """cosmo_gb300.Problem for a golden case (usdb case from the reference's own operator terms)."""
    import cosmo_gb300 as cg
    if name == "mg24usdb":
        g = golden(name)
        sps = g["sps"]
        nn = int((sps[:, 6] == 1).sum())
        return cg.Problem.from_terms(sps, nn, 4, 4, 0, 0, g["esp_keys"], g["esp_vals"], g["vspx_keys"],
                                     g["vspx_vals"])
    return cg.Problem(synthetic_xml(name, tmpdir))


@pytest.fixture(scope="session")
def gpu_available():
    import cosmo_gb300 as cg
    if cg.device_count() < 1:
        pytest.skip("no CUDA device")
    return True
