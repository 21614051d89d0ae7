"""ctypes binding of the CPU oracle (oracle/_build/liboracle.so).

TEST INFRASTRUCTURE ONLY: the FP64 restatement of the reference that the
GB300 kernels are checked against, and the timed CPU baseline.  Only tests/,
__graft_entry__.smoke() and bench.py's CPU-baseline / reference arm use it.
Parity unpinned against the reference's own outputs (the reference ships no
tests or golden outputs and cannot be compiled without a Fortran compiler);
pinned by analytic known-answer tests and the Philox4x32-10 published vectors.
"""
from __future__ import annotations

import ctypes as C
import math
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB_PATH = HERE / "_build" / "liboracle.so"


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB_PATH


_P = C.c_void_p
_f = C.POINTER(C.c_float)
_i = C.POINTER(C.c_int32)
_d = C.POINTER(C.c_double)


class TransportIn(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("n_cells", C.c_int32), ("nbins", C.c_int32),
                ("symmetric_xyz", C.c_int32), ("lg_dust", C.c_int32), ("lg_gas", C.c_int32),
                ("lg_compton", C.c_int32), ("rad_press", C.c_int32),
                ("x_axis", _P), ("y_axis", _P), ("z_axis", _P), ("active", _P), ("nu", _P), ("src_cdf", _P),
                ("kn_sigma_t", _P), ("kn_cdf", _P), ("pcomp", _P), ("opacity", _P), ("sca_opac", _P),
                ("rec_pdf", _P), ("dust_pdf", _P), ("total_lines", _P), ("ne", _P),
                ("ion_edge1", C.c_float), ("r_out", C.c_float), ("star_pos", C.c_float * 3),
                ("star_idx", C.c_int32 * 3), ("delta_e", C.c_double), ("n_angle", C.c_int32),
                ("tot_phi", C.c_int32), ("view_p_theta", C.c_int32 * 21), ("view_p_phi", C.c_int32 * 21),
                ("plane", C.c_int32)]


def view_bins(n_angle: int, theta, phi) -> tuple[int, list, list]:
    """totAngleBinsPhi, viewPointPtheta(0:20) and viewPointPphi(0:20) of initCartesianGrid
    (source/grid_mod.f90:570-601): 20 theta bins over [0, pi], 20 phi bins over [0, 2 pi), or one
    phi bin when a view's phi is negative (every view's phi is then taken as -1)."""
    pi = 3.141592654
    tot_phi = 20
    phi = [float(phi[k]) for k in range(n_angle)]
    if any(v < 0 for v in phi):
        tot_phi, phi = 1, [-1.0] * n_angle
    d_theta, d_phi = pi / 20, 2 * pi / tot_phi
    pt, pp = [0] * 21, [0] * 21
    for k in range(n_angle):
        pt[int(float(theta[k]) / d_theta) + 1] = k + 1
        pp[int(phi[k] / d_phi) + 1] = k + 1
    return tot_phi, pt, pp


class TransportOut(C.Structure):
    _fields_ = [("jste", _P), ("escaped", _P), ("h_est", _P)]


class TransportStats(C.Structure):
    _fields_ = [("crossings", C.c_int64), ("interactions", C.c_int64), ("absorptions", C.c_int64),
                ("scatterings", C.c_int64), ("escaped", C.c_int64), ("line_escapes", C.c_int64),
                ("trapped", C.c_int64), ("emissions", C.c_int64), ("q_phot", C.c_double), ("error", C.c_int32),
                ("pad", C.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "pad"}


class OpacityIn(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("nbins", C.c_int32), ("nstages", C.c_int32), ("n_elem_used", C.c_int32),
                ("lg_compton", C.c_int32), ("n_xsec", C.c_int32), ("nu", _P), ("xsec", _P), ("kn_sigma_t", _P),
                ("ptr", _P), ("elem_abun", _P), ("elem_xref", _P), ("n_shells", _P), ("element_p", _P),
                ("hden", _P), ("te", _P), ("ne", _P), ("ionden", _P), ("gaunt_te", _P), ("compute", _P)]


class EmissionIn(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("nbins", C.c_int32), ("nstages", C.c_int32), ("n_elem_used", C.c_int32),
                ("n_xsec", C.c_int32), ("n_fb_heavy", C.c_int32), ("n_tk", C.c_int32), ("nlim", C.c_int32 * 3),
                ("j2ts_p", C.c_int32), ("heii_lyman_p", C.c_int32 * 4),
                ("nu", _P), ("widflx", _P), ("xsec", _P), ("ptr", _P), ("elem_abun", _P), ("elem_xref", _P),
                ("tk", _P), ("gamma_edge_p", _P), ("log_gamma", _P), ("fb_heavy", _P), ("gaunt_ff", _P),
                ("gaunt_ff_heii", _P), ("hei2phot", _P), ("heii_lyman", _P), ("hydro_file_map", _P),
                ("hydro_dens", _P), ("hydro_lines", _P), ("hydro_temps", _P), ("hb_coeff", _P), ("rb_edge", _P),
                ("r2a_edge", _P), ("hei_rec", _P), ("te", _P), ("ne", _P), ("ionden", _P), ("for_lines", _P),
                ("compute", _P)]


_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            build()
        l = C.CDLL(str(LIB_PATH))
        l.orc_philox4x32_10.argtypes = [_P, _P, _P]
        l.orc_philox4x32_10.restype = None
        l.orc_fm_eval.argtypes = [C.c_int32, _P, _P, C.c_int64, _P]
        l.orc_fm_eval.restype = None
        l.orc_transport.argtypes = [C.POINTER(TransportIn), C.c_uint64, C.c_uint64, C.c_int64, C.c_int32,
                                    C.POINTER(TransportOut), C.POINTER(TransportStats)]
        l.orc_transport.restype = C.c_int
        l.orc_opacity.argtypes = [C.POINTER(OpacityIn), _P]
        l.orc_opacity.restype = C.c_int
        l.orc_gaunt_ff.argtypes = [C.c_double, C.c_double, _P, C.c_int32, _P]
        l.orc_gaunt_ff.restype = None
        l.orc_gaunt_cache.argtypes = [C.c_int32, C.c_int32, C.c_int32, _P, _P, _P, C.POINTER(C.c_float), _P]
        l.orc_gaunt_cache.restype = None
        l.orc_emission.argtypes = [C.POINTER(EmissionIn), _P, _P]
        l.orc_emission.restype = C.c_int
        _lib = l
    return _lib


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


def _split_mask(compute: np.ndarray, nthreads: int) -> list[np.ndarray]:
    """The cells of a compute mask cut into nthreads contiguous runs of about
    equal count (the oracle's per-cell phases then run one run per thread:
    ctypes releases the GIL for the foreign call)."""
    idx = np.nonzero(compute)[0]
    out = []
    for part in np.array_split(idx, max(1, min(nthreads, idx.size))):
        m = np.zeros_like(compute)
        m[part] = 1
        out.append(m)
    return out


def _threads(fn, masks):
    if len(masks) == 1:
        return [fn(masks[0])]
    from concurrent.futures import ThreadPoolExecutor
    with ThreadPoolExecutor(max_workers=len(masks)) as ex:
        return list(ex.map(fn, masks))


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, dtype=np.uint32)
    k = np.ascontiguousarray(key, dtype=np.uint32)
    out = np.zeros(4, dtype=np.uint32)
    lib().orc_philox4x32_10(_p(c), _p(k), _p(out))
    return out


FM_EXP, FM_LOG, FM_LOG10, FM_POW, FM_SIN, FM_COS = 0, 1, 2, 3, 4, 5


def fm_eval(fn: int, x, y=None) -> np.ndarray:
    """The portable FP64 exp / log / log10 / pow / sin / cos that the oracle
    and the device's FP64 balance and transport share, evaluated on the host."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(np.zeros_like(x) if y is None else y, dtype=np.float64)
    out = np.empty_like(x)
    lib().orc_fm_eval(fn, _p(x), _p(y), x.size, _p(out))
    return out


def gaunt_ff(z: float, log10te: float, nu: np.ndarray) -> np.ndarray:
    nu = np.ascontiguousarray(nu, dtype=np.float32)
    g = np.zeros(nu.size, dtype=np.float64)
    lib().orc_gaunt_ff(z, log10te, _p(nu), nu.size, _p(g))
    return g


def gaunt_cache(nx, ny, nz, active, te, compute, te_old: float) -> tuple[np.ndarray, float]:
    active = np.ascontiguousarray(active, dtype=np.int32)
    te = np.ascontiguousarray(te, dtype=np.float32)
    compute = np.ascontiguousarray(compute, dtype=np.uint8)
    out = np.zeros(te.size, dtype=np.float32)
    t = C.c_float(te_old)
    lib().orc_gaunt_cache(nx, ny, nz, _p(active), _p(te), _p(compute), C.byref(t), _p(out))
    return out, t.value


def opacity(setup, te=None, ne=None, ionden=None, hden=None, gaunt_te=None, compute=None, out=None,
            nthreads: int = 1) -> np.ndarray:
    """Oracle opacity for a mocassin_xray_gb300.Setup (arrays default to the set-up's state); the
    cells are shared among `nthreads` threads (each writes only its own cells)."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    C1, nb = i.n_cells + 1, i.nbins
    arrs = dict(
        nu=setup.get(abi.ARR_NU), xsec=setup.get(abi.ARR_XSEC), kn=setup.get(abi.ARR_KN_SIGMA_T),
        ptr=setup.get(abi.SARR_POINTERS), abun=setup.get(abi.ARR_ELEM_ABUN), xref=setup.get(abi.SARR_ELEM_XREF),
        nsh=setup.get(abi.SARR_N_SHELLS), ep=setup.get(abi.SARR_ELEMENT_P),
        hden=np.ascontiguousarray(hden if hden is not None else setup.get(abi.ARR_HDEN), dtype=np.float32),
        te=np.ascontiguousarray(te if te is not None else setup.get(abi.ARR_TE), dtype=np.float32),
        ne=np.ascontiguousarray(ne if ne is not None else setup.get(abi.ARR_NE), dtype=np.float32),
        ion=np.ascontiguousarray(ionden if ionden is not None else setup.get(abi.ARR_IONDEN), dtype=np.float32),
    )
    if compute is None:
        compute = np.ones(C1, dtype=np.uint8)
        compute[0] = 0
    compute = np.ascontiguousarray(compute, dtype=np.uint8)
    if gaunt_te is None:
        gaunt_te, _ = gaunt_cache(i.nx, i.ny, i.nz, setup.get(abi.ARR_ACTIVE), arrs["te"], compute, -1.0)
    gaunt_te = np.ascontiguousarray(gaunt_te, dtype=np.float32)
    if out is None:
        out = np.zeros((nb, C1), dtype=np.float32)
    def run(mask):
        s = OpacityIn(n_cells=i.n_cells, nbins=nb, nstages=i.nstages, n_elem_used=max(i.n_elem_used, 1),
                      lg_compton=i.lg_compton, n_xsec=arrs["xsec"].size, nu=_p(arrs["nu"]), xsec=_p(arrs["xsec"]),
                      kn_sigma_t=_p(arrs["kn"]), ptr=_p(arrs["ptr"]), elem_abun=_p(arrs["abun"]),
                      elem_xref=_p(arrs["xref"]), n_shells=_p(arrs["nsh"]), element_p=_p(arrs["ep"]),
                      hden=_p(arrs["hden"]), te=_p(arrs["te"]), ne=_p(arrs["ne"]), ionden=_p(arrs["ion"]),
                      gaunt_te=_p(gaunt_te), compute=_p(mask))
        return lib().orc_opacity(C.byref(s), _p(out))

    for rc in _threads(run, _split_mask(compute, nthreads)):
        if rc != 0:
            raise RuntimeError(f"orc_opacity failed: {rc}")
    return out


def transport(setup, opacity_arr, rec_pdf, total_lines, ne=None, n: int = 1000, seed: int = 0,
              counter_base: int = 0, nthreads: int = 1, n_photons_norm: int = 0,
              sca_opac=None, dust_pdf=None, istar: int = 1):
    """Oracle transport of packets [counter_base, counter_base+n) of ionising source `istar` (its
    luminosity, position and CDF: energyPacketDriver(iStar, ...), source/photon_mod.f90:28-416);
    returns (Jste, escaped, stats)."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    C1, nb = i.n_cells + 1, i.nbins
    star = setup.get(abi.SARR_STARS).reshape(-1, 8)[istar - 1]
    keep = dict(
        x=setup.get(abi.ARR_XAXIS), y=setup.get(abi.ARR_YAXIS), z=setup.get(abi.ARR_ZAXIS),
        act=setup.get(abi.ARR_ACTIVE), nu=setup.get(abi.ARR_NU),
        cdf=np.ascontiguousarray(setup.get(abi.SARR_SRC_CDFS).reshape(-1, nb)[istar - 1]),
        kn=setup.get(abi.ARR_KN_SIGMA_T), kncdf=setup.get(abi.ARR_KN_CDF), pc=setup.get(abi.ARR_PCOMP),
        op=np.ascontiguousarray(opacity_arr, dtype=np.float32),
        rec=np.ascontiguousarray(rec_pdf, dtype=np.float32),
        tl=np.ascontiguousarray(total_lines, dtype=np.float32),
        ne=np.ascontiguousarray(ne if ne is not None else setup.get(abi.ARR_NE), dtype=np.float32),
        sca=None if sca_opac is None else np.ascontiguousarray(sca_opac, dtype=np.float32),
        dust=None if dust_pdf is None else np.ascontiguousarray(dust_pdf, dtype=np.float32),
    )
    norm = n_photons_norm if n_photons_norm > 0 else n
    s = TransportIn(nx=i.nx, ny=i.ny, nz=i.nz, n_cells=i.n_cells, nbins=nb, symmetric_xyz=i.symmetric_xyz,
                    lg_dust=i.lg_dust, lg_gas=i.lg_gas, lg_compton=i.lg_compton, rad_press=0,
                    x_axis=_p(keep["x"]), y_axis=_p(keep["y"]), z_axis=_p(keep["z"]), active=_p(keep["act"]),
                    nu=_p(keep["nu"]), src_cdf=_p(keep["cdf"]), kn_sigma_t=_p(keep["kn"]),
                    kn_cdf=_p(keep["kncdf"]), pcomp=_p(keep["pc"]), opacity=_p(keep["op"]),
                    sca_opac=_p(keep["sca"]), rec_pdf=_p(keep["rec"]), dust_pdf=_p(keep["dust"]),
                    total_lines=_p(keep["tl"]), ne=_p(keep["ne"]), ion_edge1=i.ion_edge1, r_out=i.r_out,
                    delta_e=float(np.float32(star[0])) / norm)
    s.star_pos[:] = [float(v) for v in star[2:5]]
    s.star_idx[:] = [int(v) for v in star[5:8]]
    s.n_angle = i.n_angle_bins
    s.plane = i.plane_ionization
    s.tot_phi, pt, pp = view_bins(i.n_angle_bins, i.view_theta, i.view_phi)
    s.view_p_theta[:] = pt
    s.view_p_phi[:] = pp
    j = np.zeros((nb, C1), dtype=np.float64)
    e = np.zeros((nb + 1, C1) if i.n_angle_bins == 0 else (i.n_angle_bins + 1, nb + 1, C1), dtype=np.float64)
    o = TransportOut(jste=_p(j), escaped=_p(e), h_est=None)
    st = TransportStats()
    rc = lib().orc_transport(C.byref(s), seed, counter_base, n, nthreads, C.byref(o), C.byref(st))
    if rc != 0:
        raise RuntimeError(f"orc_transport failed: {rc}")
    return j, e, st


def _emission_struct(setup, te=None, ne=None, ionden=None):
    """EmissionIn for a Setup and a grid state, with the arrays it points at (keep them alive)."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    dims = setup.get(abi.SARR_EM_DIMS)
    k = dict(
        nu=setup.get(abi.ARR_NU), wid=setup.get(abi.ARR_WIDFLX), xsec=setup.get(abi.ARR_XSEC),
        ptr=setup.get(abi.SARR_POINTERS), abun=setup.get(abi.ARR_ELEM_ABUN), xref=setup.get(abi.SARR_ELEM_XREF),
        tk=setup.get(abi.SARR_EM_TK), edge=setup.get(abi.SARR_EM_EDGE_P), lg=setup.get(abi.SARR_EM_LOG_GAMMA),
        fb=setup.get(abi.SARR_EM_FB_HEAVY), h2=setup.get(abi.SARR_EM_HEI_2PHOT),
        ly=np.ascontiguousarray(setup.get(abi.SARR_EM_HEII_LYMAN)[:4]),
        hmap=setup.get(abi.SARR_EM_HYDRO_MAP), hdens=setup.get(abi.SARR_EM_HYDRO_DENS),
        hlines=setup.get(abi.SARR_EM_HYDRO_LINES), htemps=setup.get(abi.SARR_EM_HYDRO_TEMPS),
        hb=setup.get(abi.SARR_EM_HB_COEFF), rb=setup.get(abi.SARR_EM_RB_EDGE), r2a=setup.get(abi.SARR_EM_R2A_EDGE),
        heirec=setup.get(abi.SARR_EM_HEI_REC),
        te=np.ascontiguousarray(te if te is not None else setup.get(abi.ARR_TE), dtype=np.float32),
        ne=np.ascontiguousarray(ne if ne is not None else setup.get(abi.ARR_NE), dtype=np.float32),
        ion=np.ascontiguousarray(ionden if ionden is not None else setup.get(abi.ARR_IONDEN), dtype=np.float32),
    )
    s = EmissionIn(n_cells=i.n_cells, nbins=i.nbins, nstages=i.nstages, n_elem_used=max(i.n_elem_used, 1),
                   n_xsec=k["xsec"].size, n_fb_heavy=int(dims[4]), n_tk=int(dims[0]), j2ts_p=int(dims[6]))
    s.nlim[:] = [int(x) for x in dims[1:4]]
    s.heii_lyman_p[:] = [int(x) for x in dims[7:11]]
    for f, key in (("nu", "nu"), ("widflx", "wid"), ("xsec", "xsec"), ("ptr", "ptr"), ("elem_abun", "abun"),
                   ("elem_xref", "xref"), ("tk", "tk"), ("gamma_edge_p", "edge"), ("log_gamma", "lg"),
                   ("fb_heavy", "fb"), ("hei2phot", "h2"),
                   ("heii_lyman", "ly"), ("hydro_file_map", "hmap"), ("hydro_dens", "hdens"),
                   ("hydro_lines", "hlines"), ("hydro_temps", "htemps"), ("hb_coeff", "hb"), ("rb_edge", "rb"),
                   ("r2a_edge", "r2a"), ("hei_rec", "heirec"), ("te", "te"), ("ne", "ne"), ("ionden", "ion")):
        setattr(s, f, _p(k[key]))
    return s, k


def emission(setup, gaunt_te: float, te=None, ne=None, ionden=None, compute=None, for_lines=None,
             rec_pdf=None, total_lines=None, nthreads: int = 1):
    """Oracle emission phase for a mocassin_xray_gb300.Setup: returns (recPDF [nbins][C+1], totalLines [C+1]).
    `gaunt_te` is the temperature of the last Gaunt tabulation of the opacity phase; the cells are
    shared among `nthreads` threads (each writes only its own cells)."""
    i = setup.info
    C1, nb = i.n_cells + 1, i.nbins
    s, k = _emission_struct(setup, te, ne, ionden)
    nu = k["nu"]
    k["g1"] = gaunt_ff(0.0, math.log10(gaunt_te), nu).astype(np.float32)
    k["g2"] = gaunt_ff(0.30103, math.log10(gaunt_te), nu).astype(np.float32)
    s.gaunt_ff = _p(k["g1"])
    s.gaunt_ff_heii = _p(k["g2"])
    fl = None if for_lines is None else np.ascontiguousarray(for_lines, dtype=np.float32)
    if compute is None:
        compute = np.ones(C1, dtype=np.uint8)
        compute[0] = 0
    compute = np.ascontiguousarray(compute, dtype=np.uint8)
    if rec_pdf is None:
        rec_pdf = np.zeros((nb, C1), dtype=np.float32)
    if total_lines is None:
        total_lines = np.zeros(C1, dtype=np.float32)
    s.for_lines = _p(fl)

    def run(mask):
        si = EmissionIn.from_buffer_copy(s)
        si.compute = _p(mask)
        return lib().orc_emission(C.byref(si), _p(rec_pdf), _p(total_lines))

    for rc in _threads(run, _split_mask(compute, nthreads)):
        if rc != 0:
            raise RuntimeError(f"orc_emission failed: {rc}")
    return rec_pdf, total_lines


class BalanceIn(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("nbins", C.c_int32), ("nstages", C.c_int32), ("n_elem_used", C.c_int32),
                ("n_xsec", C.c_int32), ("lg_badnell", C.c_int32), ("lg_compton", C.c_int32), ("n_diel", C.c_int32),
                ("n_aldro", C.c_int32), ("n_atoms", C.c_int32), ("xhi_limit", C.c_float),
                ("nu", _P), ("xsec", _P), ("ptr", _P), ("xsec_recoil", _P), ("elem_abun", _P), ("elem_xref", _P),
                ("n_shells", _P), ("element_p", _P), ("cf", _P), ("cion_therm", _P), ("nauger", _P), ("auger", _P),
                ("rr_badnell", _P), ("dr_c", _P), ("dr_e", _P), ("rrec", _P), ("rnew", _P), ("diel", _P),
                ("aldro", _P), ("outer", _P), ("atom_index", _P), ("atom_hdr", _P), ("atom_data", _P),
                ("jste", _P), ("hden", _P)]


class BalanceState(C.Structure):
    _fields_ = [("te", _P), ("ne", _P), ("ionden", _P), ("converged", _P), ("black", _P), ("n_iter_t", _P)]


class BalanceStats(C.Structure):
    _fields_ = [("no_hit", C.c_double), ("no_ion_bal", C.c_double), ("no_te_bal", C.c_double),
                ("converged", C.c_int64)]


def _balance_lib():
    l = lib()
    if not getattr(l, "_balance_ready", False):
        l.orc_balance.argtypes = [C.POINTER(BalanceIn), C.POINTER(BalanceState), C.c_int32, C.POINTER(BalanceStats)]
        l.orc_balance.restype = C.c_int
        l.orc_equilibrium.argtypes = [C.POINTER(BalanceIn), C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int32,
                                      _P, _P]
        l.orc_equilibrium.restype = C.c_int
        l.orc_for_lines_emission.argtypes = [C.POINTER(BalanceIn), _P, _P, _P, _P, _P]
        l.orc_balance_trace.argtypes = [C.POINTER(BalanceIn), C.POINTER(BalanceState), C.c_int32, _P]
        l.orc_balance_trace.restype = C.c_int
        l.orc_balance_fixed_te.argtypes = [C.POINTER(BalanceIn), C.POINTER(BalanceState), C.c_int32, C.c_double, _P]
        l.orc_balance_fixed_te.restype = C.c_int
        l.orc_for_lines_emission.restype = C.c_int
        l._balance_ready = True
    return l


class BalanceTables:
    """The set-up tables the balance oracle reads, taken from a Setup once."""

    def __init__(self, setup, lg_badnell: bool = True):
        from mocassin_xray_gb300 import abi
        i = setup.info
        g = setup.get
        self.k = dict(
            nu=g(abi.ARR_NU), xsec=g(abi.ARR_XSEC), ptr=g(abi.SARR_POINTERS), rec=g(abi.SARR_XSEC_RECOIL),
            abun=g(abi.ARR_ELEM_ABUN), xref=g(abi.SARR_ELEM_XREF), nsh=g(abi.SARR_N_SHELLS),
            ep=g(abi.SARR_ELEMENT_P), cf=g(abi.SARR_CION_CF), ct=g(abi.SARR_CION_THERM), na=g(abi.SARR_NAUGER),
            au=g(abi.SARR_AUGER), rr=g(abi.SARR_RR_BADNELL), drc=g(abi.SARR_DR_BADNELL_C),
            dre=g(abi.SARR_DR_BADNELL_E), rrec=g(abi.SARR_RADREC_RREC), rnew=g(abi.SARR_RADREC_RNEW),
            diel=g(abi.SARR_DIELEC), aldro=g(abi.SARR_ALDRO), outer=g(abi.SARR_OUTER_SHELL),
            aidx=g(abi.SARR_ATOM_INDEX), ahdr=g(abi.SARR_ATOM_HDR), adata=g(abi.SARR_ATOM_DATA),
            hden=g(abi.ARR_HDEN))
        k = self.k
        self.info = i
        self.s = BalanceIn(n_cells=i.n_cells, nbins=i.nbins, nstages=i.nstages, n_elem_used=max(i.n_elem_used, 1),
                           n_xsec=k["xsec"].size, lg_badnell=1 if lg_badnell else 0, lg_compton=i.lg_compton,
                           n_diel=k["diel"].size // 8, n_aldro=k["aldro"].size // 6, n_atoms=k["ahdr"].size // 16,
                           xhi_limit=i.xhi_limit)
        for f, key in (("nu", "nu"), ("xsec", "xsec"), ("ptr", "ptr"), ("xsec_recoil", "rec"), ("elem_abun", "abun"),
                       ("elem_xref", "xref"), ("n_shells", "nsh"), ("element_p", "ep"), ("cf", "cf"),
                       ("cion_therm", "ct"), ("nauger", "na"), ("auger", "au"), ("rr_badnell", "rr"),
                       ("dr_c", "drc"), ("dr_e", "dre"), ("rrec", "rrec"), ("rnew", "rnew"), ("diel", "diel"),
                       ("aldro", "aldro"), ("outer", "outer"), ("atom_index", "aidx"), ("atom_hdr", "ahdr"),
                       ("atom_data", "adata"), ("hden", "hden")):
            setattr(self.s, f, _p(k[key]))

    def atom(self, elem: int, ion: int) -> int:
        return int(self.k["aidx"].reshape(30, 31)[elem - 1, ion - 1])

    def nlev(self, atom: int) -> int:
        return int(self.k["ahdr"].reshape(-1, 16)[atom, 2])


def equilibrium(tables: BalanceTables, atom: int, te: float, ne: float, ion_den_up: float = 0.0, rec: bool = False):
    """Level populations and line emissivities [lower][upper] of one ion (equilibrium)."""
    nlev = tables.nlev(atom)
    n = np.zeros(nlev, dtype=np.float64)
    em = np.zeros((nlev, nlev), dtype=np.float64)
    _balance_lib().orc_equilibrium(C.byref(tables.s), atom, te, ne, ion_den_up, 1 if rec else 0, _p(n), _p(em))
    return n, em


def balance(tables: BalanceTables, jste, te, ne, ionden, nthreads: int = 1):
    """updateCell for every cell: returns (te, ne, ionden, converged, black, n_iter_t, stats)."""
    i = tables.info
    C1 = i.n_cells + 1
    jste = np.ascontiguousarray(jste, dtype=np.float64)
    te = np.array(te, dtype=np.float32, copy=True)
    ne = np.array(ne, dtype=np.float32, copy=True)
    ionden = np.array(ionden, dtype=np.float32, copy=True).reshape(-1)
    conv = np.zeros(C1, dtype=np.int32)
    black = np.zeros(C1, dtype=np.int32)
    nit = np.zeros(C1, dtype=np.int32)
    tables.s.jste = _p(jste)
    st = BalanceState(te=_p(te), ne=_p(ne), ionden=_p(ionden), converged=_p(conv), black=_p(black),
                      n_iter_t=_p(nit))
    stats = BalanceStats()
    rc = _balance_lib().orc_balance(C.byref(tables.s), C.byref(st), nthreads, C.byref(stats))
    tables.s.jste = None
    if rc != 0:
        raise RuntimeError(f"orc_balance failed: {rc}")
    return te, ne, ionden, conv, black, nit, stats


class _Swap:
    """Points fields of a ctypes struct at other arrays for the length of a with-block."""

    def __init__(self, struct, **arrays):
        self.struct, self.arrays, self.saved = struct, arrays, {}

    def __enter__(self):
        for f, a in self.arrays.items():
            if a is not None:
                self.saved[f] = getattr(self.struct, f)
                setattr(self.struct, f, _p(a))
        return self

    def __exit__(self, *exc):
        for f, v in self.saved.items():
            setattr(self.struct, f, v)


def balance_fixed_te(tables: BalanceTables, jste, te, ne, ionden, x_tol=float(np.float32(1e-14)), hden=None,
                     abun=None, nthreads: int = 1):
    """The balance of every cell with its Te held (orc_balance_fixed_te): ionBalance converged to x_tol at
    the given Te, then heating - cooling.  hden [C+1] and abun [30] replace the set-up's densities and
    abundances.  Returns (ne, ionden, resid, converged, black, rounds)."""
    i = tables.info
    C1 = i.n_cells + 1
    jste = np.ascontiguousarray(jste, dtype=np.float64)
    te = np.array(te, dtype=np.float32, copy=True)
    ne = np.array(ne, dtype=np.float32, copy=True)
    ionden = np.array(ionden, dtype=np.float32, copy=True).reshape(-1)
    conv = np.zeros(C1, dtype=np.int32)
    black = np.zeros(C1, dtype=np.int32)
    rounds = np.zeros(C1, dtype=np.int32)
    resid = np.zeros(C1, dtype=np.float64)
    hd = None if hden is None else np.ascontiguousarray(hden, dtype=np.float32)
    ab = None if abun is None else np.ascontiguousarray(abun, dtype=np.float32)
    st = BalanceState(te=_p(te), ne=_p(ne), ionden=_p(ionden), converged=_p(conv), black=_p(black),
                      n_iter_t=_p(rounds))
    with _Swap(tables.s, jste=jste, hden=hd, elem_abun=ab):
        rc = _balance_lib().orc_balance_fixed_te(C.byref(tables.s), C.byref(st), nthreads, float(x_tol), _p(resid))
    tables.s.jste = None
    if rc != 0:
        raise RuntimeError(f"orc_balance_fixed_te failed: {rc}")
    return ne, ionden, resid, conv, black, rounds


def for_lines_emission(tables: BalanceTables, te, ne, ionden, compute=None, nthreads: int = 1) -> np.ndarray:
    """normFor of each cell (with compute[c] = 1): the emission phase's
    forbidden-line total [1e-25 erg/s per gas density]; the cells are shared
    among `nthreads` threads."""
    C1 = tables.info.n_cells + 1
    te = np.ascontiguousarray(te, dtype=np.float32)
    ne = np.ascontiguousarray(ne, dtype=np.float32)
    ionden = np.ascontiguousarray(ionden, dtype=np.float32).reshape(-1)
    comp = np.ones(C1, np.uint8) if compute is None else np.ascontiguousarray(compute, dtype=np.uint8)
    out = np.zeros(C1, dtype=np.float64)
    masks = _split_mask(comp, nthreads)

    def run(mask):
        o = np.zeros(C1, dtype=np.float64)
        _balance_lib().orc_for_lines_emission(C.byref(tables.s), _p(te), _p(ne), _p(ionden), _p(mask), _p(o))
        return mask, o

    for mask, o in _threads(run, masks):
        out[mask > 0] = o[mask > 0]
    return out


def balance_trace(tables: BalanceTables, jste, te, ne, ionden, cell: int) -> np.ndarray:
    """The T-iterations of one cell: rows of (Te, heating, cooling, Ne, X(H0))."""
    i = tables.info
    C1 = i.n_cells + 1
    jste = np.ascontiguousarray(jste, dtype=np.float64)
    te = np.array(te, dtype=np.float32, copy=True)
    ne = np.array(ne, dtype=np.float32, copy=True)
    ionden = np.array(ionden, dtype=np.float32, copy=True).reshape(-1)
    conv = np.zeros(C1, dtype=np.int32)
    black = np.zeros(C1, dtype=np.int32)
    nit = np.zeros(C1, dtype=np.int32)
    tables.s.jste = _p(jste)
    st = BalanceState(te=_p(te), ne=_p(ne), ionden=_p(ionden), converged=_p(conv), black=_p(black),
                      n_iter_t=_p(nit))
    tr = np.zeros((20, 5), dtype=np.float64)
    n = _balance_lib().orc_balance_trace(C.byref(tables.s), C.byref(st), cell, _p(tr))
    tables.s.jste = None
    return tr[:n]


class DustIn(C.Structure):
    _fields_ = [("n_cells", C.c_int32), ("nbins", C.c_int32), ("n_species", C.c_int32), ("n_sizes", C.c_int32),
                ("xhi_limit", C.c_float), ("nu", _P), ("widflx", _P), ("cabs", _P), ("csca", _P), ("abun", _P),
                ("tsub", _P), ("weight", _P), ("em_int", _P)]


class DustStats(C.Structure):
    _fields_ = [("no_hit", C.c_int64), ("updated", C.c_int64), ("converged", C.c_int64)]


class DustTables:
    """The grain tables of a dust-only Setup, for the dust oracle."""

    def __init__(self, setup):
        from mocassin_xray_gb300 import abi
        g = setup.get
        d = g(abi.SARR_DUST_DIMS)
        self.n_species, self.n_sizes = int(d[0]), int(d[1])
        self.k = dict(nu=g(abi.ARR_NU), wid=g(abi.ARR_WIDFLX), cabs=g(abi.SARR_DUST_CABS),
                      csca=g(abi.SARR_DUST_CSCA), abun=g(abi.SARR_DUST_ABUN), tsub=g(abi.SARR_DUST_TSUB),
                      weight=g(abi.SARR_DUST_WEIGHT), em=g(abi.SARR_DUST_EMINT))
        k = self.k
        i = setup.info
        self.info = i
        self.s = DustIn(n_cells=i.n_cells, nbins=i.nbins, n_species=self.n_species, n_sizes=self.n_sizes,
                        xhi_limit=i.xhi_limit, nu=_p(k["nu"]), widflx=_p(k["wid"]), cabs=_p(k["cabs"]),
                        csca=_p(k["csca"]), abun=_p(k["abun"]), tsub=_p(k["tsub"]), weight=_p(k["weight"]),
                        em_int=_p(k["em"]))


def _dust_lib():
    l = lib()
    if not getattr(l, "_dust_ready", False):
        l.orc_dust_opacity.argtypes = [C.POINTER(DustIn), _P, _P, _P, _P]
        l.orc_dust_pdf.argtypes = [C.POINTER(DustIn), _P, _P]
        l.orc_dust_t.argtypes = [C.POINTER(DustIn), _P, _P, _P, _P, C.POINTER(DustStats)]
        l._dust_ready = True
    return l


def dust_opacity(t: DustTables, ndust, tdust, opacity=None):
    C1 = t.info.n_cells + 1
    nb = t.info.nbins
    op = np.zeros((nb, C1), np.float32) if opacity is None else np.array(opacity, dtype=np.float32, copy=True)
    sca = np.zeros((nb, C1), np.float32)
    nd = np.ascontiguousarray(ndust, dtype=np.float32)
    td = np.ascontiguousarray(tdust, dtype=np.float32)
    _dust_lib().orc_dust_opacity(C.byref(t.s), _p(nd), _p(td), _p(op), _p(sca))
    return op, sca


def dust_pdf(t: DustTables, tdust):
    C1 = t.info.n_cells + 1
    pdf = np.zeros((t.info.nbins, C1), np.float32)
    td = np.ascontiguousarray(tdust, dtype=np.float32)
    _dust_lib().orc_dust_pdf(C.byref(t.s), _p(td), _p(pdf))
    return pdf


def dust_t(t: DustTables, jste, tdust):
    """getDustT: returns (tdust, converged, black, stats)."""
    C1 = t.info.n_cells + 1
    j = np.ascontiguousarray(jste, dtype=np.float64)
    td = np.array(tdust, dtype=np.float32, copy=True)
    conv = np.zeros(C1, np.int32)
    black = np.zeros(C1, np.int32)
    st = DustStats()
    _dust_lib().orc_dust_t(C.byref(t.s), _p(j), _p(td.reshape(-1)), _p(conv), _p(black), C.byref(st))
    return td, conv, black, st


def cell_volumes(setup) -> np.ndarray:
    """getVolume (source/grid_mod.f90:2887-2986) of every active cell in FP64 [e45 cm^3], [C+1]."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    keep = dict(x=setup.get(abi.ARR_XAXIS), y=setup.get(abi.ARR_YAXIS), z=setup.get(abi.ARR_ZAXIS))
    s = TransportIn(nx=i.nx, ny=i.ny, nz=i.nz, n_cells=i.n_cells, symmetric_xyz=i.symmetric_xyz,
                    x_axis=_p(keep["x"]), y_axis=_p(keep["y"]), z_axis=_p(keep["z"]))
    l = lib()
    l.orc_cell_volume.argtypes = [C.POINTER(TransportIn), C.c_int32, C.c_int32, C.c_int32]
    l.orc_cell_volume.restype = C.c_double
    act = setup.get(abi.ARR_ACTIVE).reshape(i.nz, i.ny, i.nx)
    vol = np.zeros(i.n_cells + 1, dtype=np.float64)
    for kk, jj, ii in zip(*np.nonzero(act > 0)):
        vol[act[kk, jj, ii]] = l.orc_cell_volume(C.byref(s), int(ii) + 1, int(jj) + 1, int(kk) + 1)
    return vol


class LinesOut(C.Structure):
    _fields_ = [("hbeta", C.c_double), ("hydro", _P), ("hei", _P), ("forb", _P), ("ion_num", _P),
                ("ion_den", _P), ("n_cells", C.c_int64)]


def line_luminosities(setup, tables: BalanceTables, te, ne, ionden, black, vol=None) -> dict:
    """outputGas's analytical line luminosities from a grid state (source/output_mod.f90:280-805).

    Returns hbeta_vol [1e36 erg/s] (x8 in symmetricXYZ mode), relative (lines divided by HbetaVol),
    n_cells, hydro[30,14,8] at [iz-1, iup-2, ilow-1], hei[34], forb[30, nstages, 30, 30] at
    [elem-1, ion-1, i-1, j-1] (i lower, j upper level), te_vol and ion_vol [30, nstages]."""
    i = setup.info
    S = i.nstages
    em, keep = _emission_struct(setup, te, ne, ionden)
    if vol is None:
        vol = cell_volumes(setup)
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    bl = np.ascontiguousarray(black, dtype=np.int32)
    n_atoms = tables.s.n_atoms
    hydro = np.zeros((30, 14, 8))
    hei = np.zeros(34)
    forb = np.zeros((max(n_atoms, 1), 30, 30))
    num = np.zeros((30, S))
    den = np.zeros((30, S))
    out = LinesOut(hydro=_p(hydro), hei=_p(hei), forb=_p(forb), ion_num=_p(num), ion_den=_p(den))
    l = lib()
    l.orc_line_sums.argtypes = [C.POINTER(EmissionIn), C.POINTER(BalanceIn), _P, _P, C.POINTER(LinesOut)]
    l.orc_line_sums.restype = C.c_int
    rc = l.orc_line_sums(C.byref(em), C.byref(tables.s), _p(vol), _p(bl), C.byref(out))
    if rc != 0:
        raise RuntimeError(f"orc_line_sums failed: {rc}")
    # normalisation (source/output_mod.f90:684-805)
    hb = out.hbeta
    rel = hb > 0.0
    d = hb if rel else 1.0
    forb_full = np.zeros((30, S, 30, 30))
    aidx = tables.k["aidx"].reshape(30, 31)
    for elem in range(1, 31):
        for ion in range(1, S + 1):
            a = int(aidx[elem - 1, ion - 1]) if ion <= 31 else -1
            if a >= 0:
                forb_full[elem - 1, ion - 1] = forb[a] / d
    te_vol = np.where(den > 0.0, num / np.where(den > 0.0, den, 1.0), 0.0)
    tot = den.sum(axis=1, keepdims=True)
    ion_vol = np.where(tot > 0.0, den / np.where(tot > 0.0, tot, 1.0), 0.0)
    hbv = hb * float(np.float32(1.e-16))
    if i.symmetric_xyz:
        hbv = 8.0 * hbv
    return dict(hbeta_vol=hbv, relative=bool(rel), n_cells=int(out.n_cells), hydro=hydro / d, hei=hei / d,
                forb=forb_full, te_vol=te_vol, ion_vol=ion_vol)


def line_cell_luminosities(setup, tables: BalanceTables, te, ne, ionden, cells, lines, hden=None, abun=None,
                           vol=None) -> np.ndarray:
    """[len(lines), len(cells)]: each listed cell's luminosity of the forbidden lines (elem, ion, lower,
    upper), outputGas's forbVol term of that cell alone before the division by HbetaVol
    (source/output_mod.f90:410-432), x8 in symmetricXYZ mode; hden and abun replace the set-up's."""
    i = setup.info
    C1 = i.n_cells + 1
    em, keep = _emission_struct(setup, te, ne, ionden)
    if vol is None:
        vol = cell_volumes(setup)
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    n_atoms = max(tables.s.n_atoms, 1)
    hydro, hei = np.zeros((30, 14, 8)), np.zeros(34)
    forb = np.zeros((n_atoms, 30, 30))
    num, den = np.zeros((30, i.nstages)), np.zeros((30, i.nstages))
    out = LinesOut(hydro=_p(hydro), hei=_p(hei), forb=_p(forb), ion_num=_p(num), ion_den=_p(den))
    l = lib()
    l.orc_line_sums.argtypes = [C.POINTER(EmissionIn), C.POINTER(BalanceIn), _P, _P, C.POINTER(LinesOut)]
    l.orc_line_sums.restype = C.c_int
    slots = [(tables.atom(z, ion), lo - 1, up - 1) for z, ion, lo, up in lines]
    hd = None if hden is None else np.ascontiguousarray(hden, dtype=np.float32)
    ab = None if abun is None else np.ascontiguousarray(abun, dtype=np.float32)
    res = np.zeros((len(lines), len(cells)))
    black = np.ones(C1, np.int32)
    with _Swap(tables.s, hden=hd), _Swap(em, elem_abun=ab):
        for n, cell in enumerate(cells):
            black[:] = 1
            black[int(cell)] = 0
            rc = l.orc_line_sums(C.byref(em), C.byref(tables.s), _p(vol), _p(black), C.byref(out))
            if rc != 0:
                raise RuntimeError(f"orc_line_sums failed: {rc}")
            for k, (a, lo, up) in enumerate(slots):
                res[k, n] = forb[a, lo, up]
    del keep
    return res * (8.0 if i.symmetric_xyz else 1.0)


def ift_line_gradient(setup, tables: BalanceTables, jste, te, ne, ionden, lines, cells, abun_z=(), h: float = 1e-3,
                      x_tol=float(np.float32(1e-14)), nthreads: int = 4) -> dict:
    """The implicit-function adjoint of the converged balance at fixed J, in FP64 on the CPU, for the
    listed cells: with R(Te; p) = heating - cooling of the ladder converged at Te (balance_fixed_te) and
    L(Te; p) the cell's line luminosities, the balance's root Te*(p) gives
        dL/dp = dL/dp|Te - dL/dTe|p * (dR/dp|Te) / (dR/dTe|p),
    each partial a central difference (relative step h, the stepped values rounded to FP32 as the grid
    holds them) of evaluations at Te held, started from the given converged state, their ladders
    converged to x_tol (the slow modes of the X-iteration leave a ladder stopped at 1e-9 off by up to
    1e-5, enough to spoil differences over steps of 1e-3 where dL/dp is a small difference of larger
    terms).  p is every cell's
    Hden (each cell's own; they do not interact at fixed J) and the abundances of the elements abun_z.
    Returns dL_dhden [lines, cells], dL_dabun [lines, len(abun_z), cells] (each cell's share of
    dL/d(abundance)), dte_dhden [cells], dR_dte [cells], and dL_dhden_te_held, dL_dabun_te_held (the
    partial derivatives with Te held, the gradient of a cell whose Te has no root)."""
    cells = np.asarray(cells, dtype=np.int64)
    te = np.asarray(te, np.float32)
    hden0 = tables.k["hden"].astype(np.float32)
    abun0 = tables.k["abun"].astype(np.float32)

    def evaluate(te_s, hden=None, abun=None):
        ne_s, ion_s, r, _, _, _ = balance_fixed_te(tables, jste, te_s, ne, ionden, x_tol, hden, abun, nthreads)
        lum = line_cell_luminosities(setup, tables, te_s, ne_s, ion_s, cells, lines, hden=hden, abun=abun)
        return r[cells], lum

    def central(make):
        (rp, lp, xp), (rm, lm, xm) = make(1.0 + h), make(1.0 - h)
        dx = xp - xm
        return (rp - rm) / dx, (lp - lm) / dx

    te_p = (te.astype(np.float64) * (1.0 + h)).astype(np.float32)
    te_m = (te.astype(np.float64) * (1.0 - h)).astype(np.float32)
    rt = {"p": evaluate(te_p), "m": evaluate(te_m)}
    dT = te_p[cells].astype(np.float64) - te_m[cells].astype(np.float64)
    dR_dT = (rt["p"][0] - rt["m"][0]) / dT
    dL_dT = (rt["p"][1] - rt["m"][1]) / dT

    def hden_step(f):
        hd = (hden0.astype(np.float64) * f).astype(np.float32)
        r, lum = evaluate(te, hden=hd)
        return r, lum, hd[cells].astype(np.float64)

    dR_dH, dL_dH = central(hden_step)
    dte_dh = -dR_dH / dR_dT
    out = dict(dL_dhden=dL_dH + dL_dT * dte_dh, dte_dhden=dte_dh, dR_dte=dR_dT, dL_dhden_te_held=dL_dH,
               dL_dabun=np.zeros((len(lines), len(abun_z), cells.size)),
               dL_dabun_te_held=np.zeros((len(lines), len(abun_z), cells.size)))
    for q, z in enumerate(abun_z):
        def abun_step(f, z=z):
            ab = abun0.copy()
            ab[z - 1] = np.float32(float(abun0[z - 1]) * f)
            r, lum = evaluate(te, abun=ab)
            return r, lum, np.full(cells.size, float(ab[z - 1]))
        dR_dA, dL_dA = central(abun_step)
        out["dL_dabun"][:, q, :] = dL_dA - dL_dT * dR_dA / dR_dT
        out["dL_dabun_te_held"][:, q, :] = dL_dA
    return out


def iterate_chain(setup, n_photons: int, iterations: int, seed: int, nthreads: int = 8, tables=None):
    """The loop body of iterateMC (source/iteration_mod.f90:98-1260) repeated `iterations` times from the
    set-up's initial state, all in the oracle: the skip rule of the opacity and emission loops
    (:131-149, :340-356), opacity with the Gaunt cache, emission with its forbidden lines, transport of
    the packets [(it-1)*2^40, (it-1)*2^40 + n_photons) of Philox key `seed`, J x 1e-9 (and / 8 in
    symmetricXYZ mode), then updateCell for every cell.  Returns (te, ne, ionden, black)."""
    from mocassin_xray_gb300 import abi
    i = setup.info
    C1, nb = i.n_cells + 1, i.nbins
    T = tables if tables is not None else BalanceTables(setup)
    te = setup.get(abi.ARR_TE).astype(np.float32)
    ne = setup.get(abi.ARR_NE).astype(np.float32)
    ion = setup.get(abi.ARR_IONDEN).astype(np.float32)
    te_old, ne_old = setup.get(abi.ARR_TEOLD).astype(np.float32), setup.get(abi.ARR_NEOLD).astype(np.float32)
    active = setup.get(abi.ARR_ACTIVE)
    op = np.zeros((nb, C1), np.float32)
    rec = np.zeros((nb, C1), np.float32)
    tl = np.zeros(C1, np.float32)
    gaunt_last = -1.0
    black = np.zeros(C1, np.int32)
    for it in range(1, iterations + 1):
        comp = np.ones(C1, np.uint8)
        if it > 1:
            with np.errstate(divide="ignore", invalid="ignore"):
                skip = (np.abs(te - te_old) / te_old < np.float32(0.005)) & \
                       (np.abs(ne - ne_old) / ne_old < np.float32(0.005))
            comp[skip] = 0
        comp[0] = 0
        gte, gaunt_last = gaunt_cache(i.nx, i.ny, i.nz, active, te, comp, gaunt_last)
        op = opacity(setup, te, ne, ion, gaunt_te=gte, compute=comp, out=op)
        fl = for_lines_emission(T, te, ne, ion, comp)
        rec, tl = emission(setup, gaunt_last, te, ne, ion, compute=comp, for_lines=fl, rec_pdf=rec, total_lines=tl)
        j, _, _ = transport(setup, op, rec, tl, ne=ne, n=n_photons, seed=seed, counter_base=(it - 1) << 40,
                            nthreads=nthreads)
        j = j * 1e-9
        if i.symmetric_xyz:
            j = j / 8.0
        te_old, ne_old = te.copy(), ne.copy()
        te, ne, ion, _, black, _, _ = balance(T, j, te, ne, ion, nthreads=nthreads)
        te, ne, ion = te.astype(np.float32), ne.astype(np.float32), ion.astype(np.float32)
    return te, ne, ion, black
