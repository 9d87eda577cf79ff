"""The reference's own Davidson solver driving a product through the MatrixBase
seam adapter of include/cosmo_gb300_matrix.hpp (MatrixSeam<Backend>).

The driver tests/shim/reference_davidson_seam.cpp is compiled against the
reference's kdav headers (DavidsonDiagonalization, include/kdav/davidson.cxx:
168-225; MyMatrixDiagonal, include/kdav/MandD.cxx:8-43; MatB::MatrixBase,
include/kdav/matrixbase.h:8-25) and linked with both libcosmo_gb300.so (the
GPU backend over the C ABI) and the CPU oracle.  On this CPU-only check the
product comes from the oracle's CSB, equal to the reference's own CSB product
bit for bit, so the eigenvalues the reference solver reports through the seam
must equal the ones of the reference run on its own matrix.  Needs the
reference checkout (COSMO_REFERENCE); skipped without it."""
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT, golden, manifest
from oracle import oracle as O


def _build(tmp):
    root = O.reference_root()
    if not root:
        pytest.skip("reference checkout not given (COSMO_REFERENCE)")
    import cosmo_gb300 as cg
    cg.lib()
    O.build()
    exe = os.path.join(tmp, "reference_davidson_seam")
    cmd = ["g++", "-std=c++17", "-O2", "-fopenmp", "-w", "-I", os.path.join(root, "include", "kdav"), "-I",
           os.path.join(root, "include"), "-I", os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "shim", "reference_davidson_seam.cpp"), "-o", exe,
           "-L", os.path.join(ROOT, "oracle", "_build"), "-loracle", "-L", os.path.join(ROOT, "cosmo_gb300"),
           "-lcosmo_gb300", "-Wl,-rpath," + os.path.join(ROOT, "oracle", "_build") + ":" +
           os.path.join(ROOT, "cosmo_gb300")]
    subprocess.run(cmd, check=True)
    return exe


def _read_ee(path):
    with open(path, "rb") as f:
        cnt = int(np.frombuffer(f.read(4), np.uint32)[0])
        out = []
        for _ in range(cnt):
            e, de, r = np.frombuffer(f.read(24), np.float64)
            n = int(np.frombuffer(f.read(8), np.uint64)[0])
            f.seek(8 * n, 1)
            out.append((e, de, r))
    return np.array(out)


@pytest.mark.parametrize("name", ["sd22m0s1", "sd32m1s2", "fp21m3s6"])
def test_reference_davidson_through_seam(name, tmp_path):
    exe = _build(str(tmp_path))
    g = golden(name)
    rp, c, v = (np.ascontiguousarray(g["rowptr"], np.uint64), np.ascontiguousarray(g["cols"], np.uint32),
                np.ascontiguousarray(g["vals"], np.float64))
    rows = tmp_path / "rows.bin"
    with open(rows, "wb") as f:
        f.write(np.uint64(len(rp) - 1).tobytes() + np.uint64(len(c)).tobytes())
        f.write(rp.tobytes() + c.tobytes() + v.tobytes())
    nst = len(manifest()[name]["ref_eig"])
    ee = tmp_path / "out.EE"
    subprocess.run([exe, "oracle", str(rows), str(ee), str(max(10, nst)), str(nst)], check=True,
                   stdin=subprocess.DEVNULL, capture_output=True, cwd=str(tmp_path))
    got = _read_ee(str(ee))
    assert got.shape == (nst, 3)
    np.testing.assert_allclose(got[:, 0], g["ref_eig"], rtol=0, atol=1e-10)
    np.testing.assert_allclose(got[:, 2], g["ref_resid"], rtol=1e-3, atol=1e-12)
