"""Block-tiled FP32 product (neutron-block tiles, x staged in shared memory)
against the oracle's pull-form CSB product and against the row-wise FP32
kernel.  Tolerance: 1e-5 of max|y| against the FP64 oracle (FP32 values and
vectors), 2e-6 between the two FP32 kernels (same values, different summation
order)."""
import numpy as np
import pytest

import cosmo_gb300 as cg
from conftest import problem_for
from oracle import oracle as O

pytestmark = pytest.mark.gpu

NAMES = ["sd22m0s1", "sd32m1s2", "fp21m3s6", "fp22m0s3", "sd44m0s4", "mg24usdb", "sd66m0s5"]


def _h32(name, tmp):
    """FP32 matrix with its tiled copy (built on request below 2^26 entries) and the FP64 matrix."""
    p = problem_for(name, tmp)
    b = cg.ManyBodyStates(p)
    h32 = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    h32.set_format(cg.CG_FORMAT_TILED)
    return h32, cg.Hamiltonian(p, b, cg.CG_PREC_FP64)


@pytest.mark.parametrize("name", NAMES)
def test_tiled_product_matches_oracle(gpu_available, name, tmp_path):
    h32, h64 = _h32(name, str(tmp_path))
    fmt, avail, entries = h32.format()
    assert avail and fmt == cg.CG_FORMAT_TILED
    assert entries >= h32.info.nnz_full and entries % 32 == 0
    rp, c, v = h64.upper_rows()
    for m in (8, 5):  # host blocks of 5..8 vectors are staged 8 wide -> tiled kernel
        x = np.random.default_rng(m).standard_normal((h32.n, m))
        yref = O.CSB(rp, c, v).times_matrix(x)
        scale = np.abs(yref).max()
        yt = h32.times_matrix(x, cg.CG_PREC_FP32)
        np.testing.assert_allclose(yt, yref, rtol=0, atol=1e-5 * scale)
        h32.set_format(cg.CG_FORMAT_ROWS)
        yr = h32.times_matrix(x, cg.CG_PREC_FP32)
        h32.set_format(cg.CG_FORMAT_TILED)
        np.testing.assert_allclose(yt, yr, rtol=0, atol=2e-6 * scale)


def test_tiled_built_on_request_only_below_threshold(gpu_available, tmp_path):
    p = problem_for("sd66m0s5", str(tmp_path))
    b = cg.ManyBodyStates(p)
    h = cg.Hamiltonian(p, b, cg.CG_PREC_FP32)
    assert h.info.nnz_full < 2 ** 26 and h.format()[1] is False
    h.set_format(cg.CG_FORMAT_TILED)
    assert h.format()[:2] == (cg.CG_FORMAT_TILED, True)


def test_tiled_device_call_and_format_switch(gpu_available, tmp_path):
    """cg_spmm_device with 32-byte rows (ldx = 8) through both formats."""
    torch = pytest.importorskip("torch")
    h32, h64 = _h32("sd66m0s5", str(tmp_path))
    n = h32.n
    g = torch.Generator(device="cpu").manual_seed(3)
    x = torch.randn(n, 8, generator=g, dtype=torch.float32).cuda()
    yt = torch.full((n, 8), float("nan"), dtype=torch.float32, device="cuda")
    yr = torch.full((n, 8), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    h32.spmm_device(x.data_ptr(), 8, yt.data_ptr(), 8, 8, cg.CG_PREC_FP32)
    h32.set_format(cg.CG_FORMAT_ROWS)
    assert h32.format()[0] == cg.CG_FORMAT_ROWS
    h32.spmm_device(x.data_ptr(), 8, yr.data_ptr(), 8, 8, cg.CG_PREC_FP32)
    torch.cuda.synchronize()
    a, b = yt.cpu().numpy(), yr.cpu().numpy()
    assert np.isfinite(a).all()
    np.testing.assert_allclose(a, b, rtol=0, atol=2e-6 * np.abs(b).max())
    # an FP64 matrix has no tiled copy
    assert h64.format()[1] is False
    with pytest.raises(cg.CosmoError):
        h64.set_format(cg.CG_FORMAT_TILED)


def test_tiled_autotune_reports_format(gpu_available, tmp_path):
    h32, _ = _h32("sd66m0s5", str(tmp_path))
    res = h32.autotune(nvec=8, reps=2)
    tiled = [c for c in res["candidates"] if c[1] == 0]
    assert len(tiled) == 1 and tiled[0][2] > 0
    fmt = h32.format()[0]
    best = min(res["candidates"], key=lambda c: c[2])
    assert (fmt == cg.CG_FORMAT_TILED) == (best[1] == 0)


def test_tiled_tuning_cache_roundtrip(gpu_available, tmp_path):
    """A cached choice restores the format and the tiled launch shape without timing."""
    name = "sd66m0s5"
    cache = str(tmp_path / "tune.json")
    h1, _ = _h32(name, str(tmp_path))
    r1 = h1.autotune(nvec=8, reps=2, cache=cache)
    assert r1["cached"] is False
    h2, _ = _h32(name, str(tmp_path))
    h2.set_tiled_shape(1, 2)
    h2.set_format(cg.CG_FORMAT_ROWS)
    r2 = h2.autotune(nvec=8, reps=2, cache=cache)
    assert r2["cached"] is True and r2["format"] == r1["format"]
    f1, f2 = h1.format_info(), h2.format_info()
    assert (f1["slices_per_warp"], f1["stages"]) == (f2["slices_per_warp"], f2["stages"])
    assert h1.tuning()[:2] == h2.tuning()[:2]
