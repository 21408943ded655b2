"""The sine transforms as BF16x3 tensor-core GEMMs (csrc/sgemm.cu), through the C ABI.

* ``ib_op_sine_lines_tc`` against the FP64 DST-I (scipy's RODFT00 convention halved): relative
  L2 error per line <= 5e-5 (the split keeps ~16 significant bits of each factor; the measured
  error is ~1e-5);
* the mixed-precision step with every transform on the tensor cores (precision "mixed_tc")
  against the FP64 oracle: vorticity <= 1e-8 relative L2 and C_L / C_D <= 1e-6 per step, the
  bars of the other mixed-precision paths (the refinement sweeps remove the split error).
"""
import ctypes

import numpy as np
import pytest
from scipy import fft as sfft

from _util import Dev, rel, start_pair

pytestmark = pytest.mark.gpu

LINE_TOL = 5e-5


def _handle(ib, nx, ny, precision="fp64"):
    h = 4.0 / nx
    grid = ib.MultiLevel(ib.UniformGrid(h, (-1.0, -1.0 + nx * h), (-0.5 * ny * h, 0.5 * ny * h)), 2)
    prob = ib.Problem(ib.StreamFcnFluid(grid, (1.0, 0.0), 100.0), ib.BodyGroup(), ib.SchemeCNAB(0.01))
    return ib.initsolver(prob, ib.initstate(prob), precision=precision)


@pytest.mark.parametrize("n", [128, 256, 384, 512, 768, 1024, 2048])
def test_sine_lines_match_fp64_dst(ib, lib, n):
    torch = pytest.importorskip("torch")
    s = _handle(ib, n, 128)
    rows = 300 if n <= 1024 else 260          # not a multiple of the 128-line tile
    rng = np.random.default_rng(n)
    x = rng.standard_normal((rows, n - 1)).astype(np.float32)
    x[7] *= 1e-6                                # a line far below the others' scale
    x[11, ::3] = 0.0
    d = Dev()
    xin = torch.from_numpy(x.reshape(-1)).cuda()
    out = torch.full((rows * (n - 1),), float("nan"), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for call in range(2):                       # a second call reuses the built tables
        assert lib.ib_op_sine_lines_tc(s.handle, 0, rows, ctypes.c_void_p(xin.data_ptr()),
                                       ctypes.c_void_p(out.data_ptr())) == 0
    got = d.get(out).reshape(rows, n - 1).astype(np.float64)
    want = 0.5 * sfft.dst(x.astype(np.float64), type=1, axis=-1)
    err = np.linalg.norm(got - want, axis=1) / np.linalg.norm(want, axis=1)
    assert np.all(np.isfinite(got))
    assert err.max() < LINE_TOL, (n, err.max())
    # the y axis of the same handle (n = 128) through its own table
    assert lib.ib_op_sine_lines_tc(s.handle, 1, rows, ctypes.c_void_p(xin.data_ptr()),
                                   ctypes.c_void_p(out.data_ptr())) == 0
    got_y = d.get(out).reshape(-1)[: rows * 127].reshape(rows, 127).astype(np.float64)
    xy = x.reshape(-1)[: rows * 127].reshape(rows, 127).astype(np.float64)
    want_y = 0.5 * sfft.dst(xy, type=1, axis=-1)
    assert (np.linalg.norm(got_y - want_y, axis=1) / np.linalg.norm(want_y, axis=1)).max() < LINE_TOL
    s.close()


def test_unsupported_axis_is_refused(ib, lib):
    s = _handle(ib, 192, 128)                   # 192 is not a multiple of 128
    assert lib.ib_op_sine_lines_tc(s.handle, 0, 4, None, None) != 0
    s.close()
    with pytest.raises(Exception):
        _handle(ib, 192, 128, precision="mixed_tc")


def test_info_reports_tensor_form(ib, lib):
    from ibgb300 import _lib as L
    s = _handle(ib, 256, 256, precision="mixed_tc")
    info = L.IbInfo()
    assert lib.ib_get_info(s.handle, ctypes.byref(info)) == 0
    assert info.transform_form == L.IB_FORM_TENSOR
    assert info.vort2flux_order == L.IB_V2F_SEQUENTIAL
    s.close()


@pytest.mark.parametrize("nx,ny,L,nsteps", [(128, 128, 2, 12), (256, 256, 3, 10)])
def test_tensor_core_step_parity(ib, O, nx, ny, L, nsteps):
    wl = ib.workloads.scaled(ib.workloads.two_body_large(), nx, ny, nlevels=L)
    prob, st, solver, op, ost, osol = start_pair(ib, O, wl, precision="mixed_tc")
    g = op.grid
    worst_g = worst_c = 0.0
    for i in range(nsteps):
        t = i * wl.dt
        ib.advance_(st, solver, t)
        osol.advance(ost, t)
        stress = st.qty.stress
        for k, b in enumerate(stress):
            worst_c = max(worst_c, abs(b.CD - ost.cd[k]) / max(1.0, abs(ost.cd[k])),
                          abs(b.CL - ost.cl[k]) / max(1.0, abs(ost.cl[k])))
        worst_g = max(worst_g, rel(st.qty.gamma, ost.gamma.reshape(g.nlevels, -1)))
    solver.close()
    print(f"mixed_tc {nx}x{ny}x{L}: worst gamma {worst_g:.2e}, C {worst_c:.2e}")
    assert worst_g < 1e-8 and worst_c < 1e-6, (worst_g, worst_c)
