"""mcx_transport_noalloc: the transport for callers that cannot allocate
device memory (they hand in buffers from their own pool).  It must give the
same estimators as the allocating entry point mcx_transport on the same
inputs, call after call, while keeping its scratch in the library's fixed
device array.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from conftest import synthetic_recpdf
from mocassin_xray_gb300 import abi, Context, Setup

pytestmark = pytest.mark.gpu


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def _noalloc_args(torch, s, op, rec, tl, keep):
    i = s.info
    arrs = {
        "x_axis": s.get(abi.ARR_XAXIS), "y_axis": s.get(abi.ARR_YAXIS), "z_axis": s.get(abi.ARR_ZAXIS),
        "active": s.get(abi.ARR_ACTIVE), "nu": s.get(abi.ARR_NU), "src_cdf": s.get(abi.ARR_SRC_CDF),
        "kn_sigma_t": s.get(abi.ARR_KN_SIGMA_T), "kn_cdf": s.get(abi.ARR_KN_CDF), "pcomp": s.get(abi.ARR_PCOMP),
        "opacity": op, "rec_pdf": rec, "total_lines": tl, "ne": s.get(abi.ARR_NE),
    }
    a = abi.NoallocTransportArgs()
    a.nx, a.ny, a.nz, a.n_cells, a.nbins = i.nx, i.ny, i.nz, i.n_cells, i.nbins
    a.symmetric_xyz, a.lg_compton = i.symmetric_xyz, i.lg_compton
    a.star_idx[:] = list(i.star_idx)
    a.star_pos[:] = list(i.star_pos)
    a.ion_edge1, a.r_out = i.ion_edge1, i.r_out
    for k, v in arrs.items():
        t = _dev(torch, v)
        keep.append(t)
        setattr(a, k, t.data_ptr())
    C1, nb = i.n_cells + 1, i.nbins
    j = torch.zeros((nb, C1), dtype=torch.float64, device="cuda")
    e = torch.zeros((nb + 1, C1), dtype=torch.float64, device="cuda")
    keep += [j, e]
    a.jste, a.escaped = j.data_ptr(), e.data_ptr()
    a.stream = None
    return a, j, e


def _call(a, n, seed, precision, delta_e):
    a.n_packets, a.seed, a.counter_base, a.precision = n, seed, 0, precision
    a.zero_estimators, a.delta_e = 1, delta_e
    st = abi.TransportStats()
    rc = abi.lib().mcx_transport_noalloc(ctypes.byref(a), ctypes.byref(st))
    assert rc == 0, abi.lib().mcx_noalloc_last_error().decode()
    return st


@pytest.mark.parametrize("name", ["h_small", "lognormal_small"])
def test_noalloc_matches_allocating_transport(decks, data_dir, oracle_lib, name):
    torch = pytest.importorskip("torch")
    s = Setup(decks[name], data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.full(s.n_cells + 1, 0.3, np.float32)
    ctx = Context(0)
    ctx.load(s)
    ctx.put(abi.ARR_OPACITY, op)
    ctx.put(abi.ARR_RECPDF, rec)
    ctx.put(abi.ARR_TOTAL_LINES, tl)
    keep = []
    a, j_dev, e_dev = _noalloc_args(torch, s, op, rec, tl, keep)
    torch.cuda.synchronize()
    n = 20000
    delta_e = float(np.float32(s.info.l_star)) / n
    # two calls in a row (different seeds and precisions): the shared scratch is re-cleared each call
    for seed, prec in ((11, abi.PREC_FP64), (12, abi.PREC_FP32_GEOM)):
        st_ref = ctx.transport(n, seed=seed, precision=prec)
        j_ref, e_ref = ctx.get(abi.ARR_JSTE), ctx.get(abi.ARR_ESCAPED)
        st = _call(a, n, seed, prec, delta_e)
        j, e = j_dev.cpu().numpy(), e_dev.cpu().numpy()
        for k in ("crossings", "interactions", "absorptions", "scatterings", "escaped", "line_escapes", "emissions"):
            assert getattr(st, k) == getattr(st_ref, k), k
        np.testing.assert_allclose(j, j_ref, rtol=1e-11, atol=1e-300)
        np.testing.assert_allclose(e, e_ref, rtol=1e-11, atol=1e-300)
    ctx.close()


def test_noalloc_rejects_problems_beyond_its_scratch():
    a = abi.NoallocTransportArgs()
    a.nx = a.ny = a.nz = 101
    a.n_cells, a.nbins = 101 ** 3, 1311          # ~5.4 GB of CDF rows: far above the fixed scratch
    a.star_idx[:] = [1, 1, 1]
    for k in ("x_axis", "y_axis", "z_axis", "active", "nu", "src_cdf", "kn_sigma_t", "kn_cdf", "pcomp",
              "opacity", "rec_pdf", "total_lines", "ne", "jste", "escaped"):
        setattr(a, k, 0x1000)   # never dereferenced: the size check comes first
    st = abi.TransportStats()
    rc = abi.lib().mcx_transport_noalloc(ctypes.byref(a), ctypes.byref(st))
    assert rc == 1
    assert b"scratch" in abi.lib().mcx_noalloc_last_error()


def test_noalloc_rejects_an_active_map_beyond_n_cells(decks, data_dir, oracle_lib):
    """The caller's active map is checked on the device before any packet
    moves: a voxel naming a cell above n_cells is refused (the allocating entry
    point validates the map at load time; this one never sees a load)."""
    torch = pytest.importorskip("torch")
    s = Setup(decks["h_small"], data_dir)
    op = oracle_lib.opacity(s)
    rec = synthetic_recpdf(s.get(abi.ARR_NU), s.n_cells)
    tl = np.full(s.n_cells + 1, 0.3, np.float32)
    keep = []
    a, j_dev, e_dev = _noalloc_args(torch, s, op, rec, tl, keep)
    act = s.get(abi.ARR_ACTIVE).copy()
    act.reshape(-1)[np.argmax(act.reshape(-1) > 0)] = s.n_cells + 5
    bad = _dev(torch, act)
    keep.append(bad)
    a.active = bad.data_ptr()
    torch.cuda.synchronize()
    a.n_packets, a.seed, a.counter_base, a.precision = 1000, 1, 0, abi.PREC_FP64
    a.zero_estimators, a.delta_e = 1, 1.0
    st = abi.TransportStats()
    rc = abi.lib().mcx_transport_noalloc(ctypes.byref(a), ctypes.byref(st))
    assert rc == 1                                 # MCX_ERR_INPUT
    assert b"active map" in abi.lib().mcx_noalloc_last_error()
    assert float(j_dev.abs().sum()) == 0.0        # nothing was transported
