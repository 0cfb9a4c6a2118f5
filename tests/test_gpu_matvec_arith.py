"""Arithmetic variants of the H-matvec on complex-FP32 storage: the two-float
product (refinement residual) must match FP64 arithmetic on the same stored
entries to ~1e-13; the FP32 product (inner GMRES operator) to ~1e-6."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_matvec_arithmetic_variants(bem, meshes):
    torch = pytest.importorskip("torch")
    tri = meshes.icosphere(4, 1.0)
    n = tri.shape[0]
    s = bem.Solver(aca_tol=1e-5, precision=1)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    s.assemble(1200.0)
    L = bem.lib()
    rng = np.random.default_rng(3)
    for R in (1, 3, 6):
        xh = rng.standard_normal((R, n)) + 1j * rng.standard_normal((R, n))
        x = torch.from_numpy(xh).to("cuda")
        out = {}
        for arith in (bem.BEM_ARITH_FP64, bem.BEM_ARITH_FP32, bem.BEM_ARITH_TWOFLOAT):
            y = torch.zeros((R, n), dtype=torch.complex128, device="cuda")
            st = L.bem_hmatvec_device_ex(s._h, 1, x.data_ptr(), y.data_ptr(), R, 0, arith)
            assert st == bem.BEM_OK
            torch.cuda.synchronize()
            out[arith] = y.cpu().numpy()
        ref = out[bem.BEM_ARITH_FP64]
        e2 = np.linalg.norm(out[bem.BEM_ARITH_TWOFLOAT] - ref) / np.linalg.norm(ref)
        e1 = np.linalg.norm(out[bem.BEM_ARITH_FP32] - ref) / np.linalg.norm(ref)
        assert e2 < 1e-13, (R, e2)
        assert e1 < 1e-6, (R, e1)
    y = torch.zeros(n, dtype=torch.complex128, device="cuda")
    assert L.bem_hmatvec_device_ex(s._h, 1, x.data_ptr(), y.data_ptr(), 1, 0, 7) == bem.BEM_EINVAL
    s.close()
