"""bem_hmatvec_noalloc: the H-matvec for callers that must not allocate GPU
memory during the call (real-time loops that forbid allocator calls, which can
synchronise the device; hosts whose GPU memory comes from an outside pool). It
keeps its per-block projections in a fixed device array inside the library
instead of a cudaMalloc'd buffer.

The test calls it through the C ABI twice in a row (the second call reuses the
array the first one left behind) and compares each result with the
allocating entry point bem_hmatvec_device on the same inputs. This file is
collected last so a failure here cannot hide any other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-13  # the H-matvec tolerance of the other GPU tests


@pytest.mark.parametrize("precision", [0, 1])
def test_noalloc_matches_allocating_hmatvec(bem, meshes, precision):
    torch = pytest.importorskip("torch")
    tri = meshes.icosphere(3, 1.0)
    n = tri.shape[0]
    s = bem.Solver(aca_tol=1e-5, precision=precision)
    s.set_mesh(tri)
    s.set_bc(np.zeros(n), np.ones(n))
    s.assemble(400.0)
    L = bem.lib()
    rng = np.random.default_rng(11)
    for call in range(2):
        R = 3 if call == 0 else 1
        xh = rng.standard_normal((R, n)) + 1j * rng.standard_normal((R, n))
        x = torch.from_numpy(xh.astype(np.complex128)).to("cuda")
        y_ref = torch.zeros((R, n), dtype=torch.complex128, device="cuda")
        y_new = torch.full((R, n), 7.0 + 0j, dtype=torch.complex128, device="cuda")
        st = L.bem_hmatvec_device(s._h, 1, x.data_ptr(), y_ref.data_ptr(), R, 0)
        assert st == bem.BEM_OK
        st = L.bem_hmatvec_noalloc(s._h, 1, x.data_ptr(), y_new.data_ptr(), R, 0)
        assert st == bem.BEM_OK, L.bem_last_error(s._h)
        torch.cuda.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.linalg.norm(a - b) / np.linalg.norm(b) < TOL
    # accumulate mode adds onto y
    y0 = torch.ones(n, dtype=torch.complex128, device="cuda")
    x1 = torch.from_numpy(rng.standard_normal(n) + 0j).to("cuda")
    y_ref = y0.clone()
    y_new = y0.clone()
    assert L.bem_hmatvec_device(s._h, 0, x1.data_ptr(), y_ref.data_ptr(), 1, 1) == bem.BEM_OK
    assert L.bem_hmatvec_noalloc(s._h, 0, x1.data_ptr(), y_new.data_ptr(), 1, 1) == bem.BEM_OK
    torch.cuda.synchronize()
    a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(b) < TOL
    # bad arguments are rejected with a status, not a fault
    assert L.bem_hmatvec_noalloc(s._h, 5, x1.data_ptr(), y_new.data_ptr(), 1, 0) == bem.BEM_EINVAL
    s.close()
