"""The allocation-free Laplacian inverse (ib_op_laplacian_inv_noalloc) against the allocating one.

Callers whose device memory belongs to another allocator, or whose loop cannot afford an
allocation's device-wide synchronisation, use the variant whose work buffer is a fixed array
inside the library.  It must give the same result as ib_op_laplacian_inv, call after call
(the fixed array keeps the previous call's contents), and refuse work larger than the array.
This file is collected last so a stop-at-first-failure run has already run every other test.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative L2, the operator tolerance of the other FP64 Poisson tests


def _handle(ib, nx, ny, precision="fp64"):
    h = 4.0 / nx
    grid = ib.MultiLevel(ib.UniformGrid(h, (-1.0, -1.0 + nx * h), (-0.5 * ny * h, 0.5 * ny * h)), 2)
    prob = ib.Problem(ib.StreamFcnFluid(grid, (1.0, 0.0), 100.0), ib.BodyGroup(), ib.SchemeCNAB(0.01))
    return ib.initsolver(prob, ib.initstate(prob), precision=precision)


# (grid, precision): an FP64 handle on the Stockham passes, and a mixed-precision handle, whose
# FP64 operator entry points run the warp-per-line passes
@pytest.mark.parametrize("nx,ny,precision", [(256, 192, "fp64"), (256, 256, "mixed")])
def test_noalloc_laplacian_inverse_matches_allocating_entry(ib, lib, nx, ny, precision):
    torch = pytest.importorskip("torch")
    import ctypes

    def p(t):
        return ctypes.c_void_p(t.data_ptr())

    s = _handle(ib, nx, ny, precision)
    ng = (nx - 1) * (ny - 1)
    rng = np.random.default_rng(42)
    for call in range(2):  # two calls in a row: the fixed work array holds the previous one's data
        batch = 3 - call
        b = torch.from_numpy(rng.standard_normal(batch * ng)).cuda()
        want = torch.zeros_like(b)
        got = torch.full_like(b, float("nan"))
        torch.cuda.synchronize()
        assert lib.ib_op_laplacian_inv(s.handle, batch, p(b), p(want)) == 0
        assert lib.ib_op_laplacian_inv_noalloc(s.handle, batch, p(b), p(got)) == 0
        torch.cuda.synchronize()
        w, g = want.cpu().numpy(), got.cpu().numpy()
        assert np.all(np.isfinite(g))
        assert np.linalg.norm(g - w) / np.linalg.norm(w) < TOL
    # more values than the fixed work array holds: refused with a message, nothing launched
    too_many = (1 << 22) // ng + 1
    assert lib.ib_op_laplacian_inv_noalloc(s.handle, too_many, p(b), p(got)) == 1
    assert b"exceeds" in lib.ib_last_error(s.handle)
    s.close()
