"""ctypes binding of libmcx.so (the C ABI declared in include/mcx.h).

This is the Python side of the drop-in boundary: the same entry points a
Fortran driver binds through ISO_C_BINDING.  Loading fails loudly when the
library has not been built; there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libmcx.so"

MCX_OK = 0
ERRORS = {1: "MCX_ERR_INPUT", 2: "MCX_ERR_IO", 3: "MCX_ERR_CUDA", 4: "MCX_ERR_NOMEM", 5: "MCX_ERR_STATE",
          6: "MCX_ERR_STEP_LIMIT", 7: "MCX_ERR_TIMEOUT", 8: "MCX_ERR_INTERNAL"}

# array ids (enum mcx_array_id)
(ARR_NU, ARR_WIDFLX, ARR_XSEC, ARR_SRC_CDF, ARR_KN_SIGMA_T, ARR_KN_CDF, ARR_PCOMP, ARR_XAXIS, ARR_YAXIS,
 ARR_ZAXIS, ARR_ACTIVE, ARR_HDEN, ARR_TE, ARR_NE, ARR_TEOLD, ARR_NEOLD, ARR_IONDEN, ARR_OPACITY, ARR_RECPDF,
 ARR_TOTAL_LINES, ARR_JSTE, ARR_ESCAPED, ARR_VOLUME, ARR_ELEM_ABUN, ARR_GAUNT_TE, ARR_SCAOPAC, ARR_DUSTPDF,
 ARR_NDUST, ARR_LG_CONVERGED, ARR_H_EST, ARR_LG_BLACK, ARR_N_ITER_T, ARR_FOR_LINES, ARR_TDUST,
 ARR_BAL_RESID) = range(1, 36)
SARR_POINTERS, SARR_ELEMENT_P, SARR_N_SHELLS, SARR_ELEM_XREF, SARR_ION_EDGE, SARR_COMXSEC_H, \
    SARR_COMXSEC_C, SARR_XSEC_RECOIL = range(1001, 1009)
(SARR_EM_DIMS, SARR_EM_TK, SARR_EM_EDGE_P, SARR_EM_LOG_GAMMA, SARR_EM_FB_HEAVY, SARR_EM_HYDRO_MAP,
 SARR_EM_HYDRO_DENS, SARR_EM_HYDRO_LINES, SARR_EM_HYDRO_TEMPS, SARR_EM_HB_COEFF, SARR_EM_RB_EDGE,
 SARR_EM_R2A_EDGE, SARR_EM_HEI_REC, SARR_EM_HEI_2PHOT, SARR_EM_HEII_LYMAN) = range(1009, 1024)
(SARR_CION_CF, SARR_CION_THERM, SARR_NAUGER, SARR_AUGER, SARR_RR_BADNELL, SARR_DR_BADNELL_C,
 SARR_DR_BADNELL_E, SARR_RADREC_RREC, SARR_RADREC_RNEW, SARR_DIELEC, SARR_ALDRO, SARR_OUTER_SHELL,
 SARR_ATOM_INDEX, SARR_ATOM_HDR, SARR_ATOM_DATA) = range(1024, 1039)
(SARR_DUST_DIMS, SARR_DUST_CABS, SARR_DUST_CSCA, SARR_DUST_CTABS, SARR_DUST_CTSCA, SARR_DUST_ABUN, SARR_DUST_TSUB,
 SARR_DUST_RADIUS, SARR_DUST_WEIGHT, SARR_DUST_EMINT) = range(1039, 1049)
SARR_STARS, SARR_SRC_CDFS = 1049, 1050
INT_SARR = {SARR_POINTERS, SARR_ELEMENT_P, SARR_N_SHELLS, SARR_ELEM_XREF, SARR_EM_DIMS, SARR_EM_EDGE_P,
            SARR_EM_FB_HEAVY, SARR_EM_HYDRO_MAP, SARR_NAUGER, SARR_OUTER_SHELL, SARR_ATOM_INDEX, SARR_ATOM_HDR,
            SARR_DUST_DIMS}
F64_SARR = {SARR_ATOM_DATA}
# packed atom header fields (MCX_SARR_ATOM_HDR)
(AT_ELEM, AT_ION, AT_NLEV, AT_NTEMP, AT_IUP2P, AT_RECTYPE, AT_NREC, AT_OFF_LOGT, AT_OFF_QOM, AT_OFF_Y2,
 AT_OFF_A, AT_OFF_G, AT_OFF_E, AT_OFF_REC, AT_OFF_ATP) = range(15)

MESH_REFERENCE, MESH_LOG_EDGES = 0, 1
PREC_FP32_GEOM, PREC_FP64 = 0, 1
BAL_FP64, BAL_MIXED = 0, 1
PHASE_EXACT, PHASE_MIXED = 0, 1


class SetupOpts(C.Structure):
    _fields_ = [("mesh_mode", C.c_int32), ("reserved", C.c_int32 * 7)]


class SetupInfo(C.Structure):
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("n_cells", C.c_int32),
                ("nbins", C.c_int32), ("n_xsec", C.c_int32), ("n_elem_used", C.c_int32), ("nstages", C.c_int32),
                ("symmetric_xyz", C.c_int32), ("lg_gas", C.c_int32), ("lg_dust", C.c_int32),
                ("lg_compton", C.c_int32), ("star_idx", C.c_int32 * 3), ("lyman_p", C.c_int32),
                ("n_photons", C.c_int64), ("max_iterate_mc", C.c_int32), ("n_species", C.c_int32),
                ("n_sizes", C.c_int32), ("star_pos", C.c_float * 3), ("r_out", C.c_float), ("r_in", C.c_float),
                ("l_star", C.c_float), ("l_phot", C.c_float), ("ion_edge1", C.c_float), ("te_start", C.c_float),
                ("min_convergence", C.c_float), ("xhi_limit", C.c_float), ("n_angle_bins", C.c_int32),
                ("view_theta", C.c_float * 2), ("view_phi", C.c_float * 2), ("plane_ionization", C.c_int32),
                ("n_stars", C.c_int32), ("reserved", C.c_int32 * 1)]


class BalanceOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("max_rounds", C.c_int32), ("atom_solves", C.c_int32),
                ("converge", C.c_int32), ("fix_te", C.c_int32), ("reserved", C.c_int32 * 3)]


class BalanceStats(C.Structure):
    _fields_ = [("cells_updated", C.c_int64), ("no_hit", C.c_int64), ("no_ion_bal", C.c_int64),
                ("no_te_bal", C.c_int64), ("converged", C.c_int64), ("max_iter_t", C.c_int32),
                ("kernel_ms", C.c_float), ("reserved", C.c_int64 * 4)]


class IterateOpts(C.Structure):
    _fields_ = [("n_iterate_mc", C.c_int32), ("transport_precision", C.c_int32), ("balance_precision", C.c_int32),
                ("emission_precision", C.c_int32), ("n_packets", C.c_int64), ("seed", C.c_uint64),
                ("counter_base", C.c_uint64), ("transport_block_size", C.c_int32),
                ("transport_grid_mult", C.c_int32), ("transport_emit_batch", C.c_int32),
                ("reserved", C.c_int32 * 5)]


class PhaseOpts(C.Structure):
    _fields_ = [("n_iterate_mc", C.c_int32), ("precision", C.c_int32), ("reserved", C.c_int32 * 6)]


class PhaseStats(C.Structure):
    _fields_ = [("cells_computed", C.c_int64), ("cells_skipped", C.c_int64), ("kernel_ms", C.c_float),
                ("reserved_f", C.c_float * 3), ("reserved", C.c_int64 * 4)]


class TransportOpts(C.Structure):
    _fields_ = [("istar", C.c_int32), ("precision", C.c_int32), ("n_packets", C.c_int64), ("seed", C.c_uint64),
                ("counter_base", C.c_uint64), ("n_photons_norm", C.c_int64), ("zero_estimators", C.c_int32),
                ("block_size", C.c_int32), ("grid_mult", C.c_int32), ("chunk", C.c_int32),
                ("emit_batch", C.c_int32), ("handoff_emissions", C.c_int32), ("reserved", C.c_int32 * 2)]


class TransportStats(C.Structure):
    _fields_ = [("crossings", C.c_int64), ("interactions", C.c_int64), ("absorptions", C.c_int64),
                ("scatterings", C.c_int64), ("escaped", C.c_int64), ("line_escapes", C.c_int64),
                ("trapped", C.c_int64), ("emissions", C.c_int64), ("q_phot", C.c_double), ("kernel_ms", C.c_float),
                ("reserved_f", C.c_float * 3), ("handed_off", C.c_int64), ("reserved", C.c_int64 * 3)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("reserved")}


class NoallocTransportArgs(C.Structure):
    """mcx_noalloc_transport_args: every buffer is a caller-owned device pointer."""
    _fields_ = [("nx", C.c_int32), ("ny", C.c_int32), ("nz", C.c_int32), ("n_cells", C.c_int32),
                ("nbins", C.c_int32), ("symmetric_xyz", C.c_int32), ("lg_compton", C.c_int32),
                ("precision", C.c_int32), ("star_idx", C.c_int32 * 3), ("zero_estimators", C.c_int32),
                ("star_pos", C.c_float * 3), ("ion_edge1", C.c_float), ("r_out", C.c_float), ("pad0", C.c_int32),
                ("delta_e", C.c_double), ("n_packets", C.c_int64), ("seed", C.c_uint64), ("counter_base", C.c_uint64),
                ("x_axis", C.c_void_p), ("y_axis", C.c_void_p), ("z_axis", C.c_void_p), ("active", C.c_void_p),
                ("nu", C.c_void_p), ("src_cdf", C.c_void_p), ("kn_sigma_t", C.c_void_p), ("kn_cdf", C.c_void_p),
                ("pcomp", C.c_void_p), ("opacity", C.c_void_p), ("rec_pdf", C.c_void_p),
                ("total_lines", C.c_void_p), ("ne", C.c_void_p), ("jste", C.c_void_p), ("escaped", C.c_void_p),
                ("stream", C.c_void_p)]


NOALLOC_SCRATCH_BYTES = 64 * 1024 * 1024

# exported symbols and their signatures: (name, restype, argtypes)
_P = C.c_void_p
class IterateStats(C.Structure):
    _fields_ = [("opacity", PhaseStats), ("emission", PhaseStats), ("transport", TransportStats),
                ("balance", BalanceStats), ("total_ms", C.c_float), ("reserved_f", C.c_float * 3),
                ("reserved", C.c_int64 * 4)]


class BatchPackets(C.Structure):
    _fields_ = [("n_packets", _P), ("seed", _P), ("counter_base", _P), ("n_photons_norm", _P)]


class LineRef(C.Structure):
    _fields_ = [("elem", C.c_int32), ("ion", C.c_int32), ("lower", C.c_int32), ("upper", C.c_int32)]


class SensOpts(C.Structure):
    _fields_ = [("n_lines", C.c_int32), ("n_abun", C.c_int32), ("lines", _P), ("abun_z", _P), ("h", C.c_double),
                ("precision", C.c_int32), ("reference_stopping", C.c_int32), ("reserved", C.c_int32 * 4)]


class AdjointOut(C.Structure):
    _fields_ = [("L", _P), ("dL_dhden", _P), ("dL_dabun", _P), ("dte_dhden", _P), ("kernel_ms", C.c_float),
                ("reserved_f", C.c_float * 3), ("pinned_cells", C.c_int64), ("no_solution_cells", C.c_int64),
                ("reserved", C.c_int64 * 2)]


class SensOut(C.Structure):
    _fields_ = [("L", _P), ("dL_dhden", _P), ("dL_dabun", _P), ("kernel_ms", C.c_float),
                ("reserved_f", C.c_float * 3), ("branch_cells_hden", C.c_int64), ("branch_cells_abun", C.c_int64),
                ("reserved", C.c_int64 * 2)]


class Lines(C.Structure):
    _fields_ = [("hbeta_vol", C.c_double), ("relative", C.c_int32), ("n_cells", C.c_int32),
                ("hydro_vol", _P), ("hei_vol", _P), ("forb_vol", _P), ("wav", _P), ("te_vol", _P),
                ("ion_vol", _P), ("kernel_ms", C.c_float), ("reserved_f", C.c_float * 3),
                ("reserved", C.c_int64 * 4)]


SIGNATURES = [
    ("mcx_setup_from_input", C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(SetupOpts), C.POINTER(_P)]),
    ("mcx_setup_free", None, [_P]),
    ("mcx_setup_info_get", C.c_int, [_P, C.POINTER(SetupInfo)]),
    ("mcx_setup_get", C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    ("mcx_setup_len", C.c_int, [_P, C.c_int32, C.POINTER(C.c_int64)]),
    ("mcx_setup_set", C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    ("mcx_setup_last_error", C.c_char_p, []),
    ("mcx_ctx_create", C.c_int, [C.c_int32, C.POINTER(_P)]),
    ("mcx_ctx_destroy", None, [_P]),
    ("mcx_last_error", C.c_int, [_P, C.c_char_p, C.c_size_t]),
    ("mcx_sync", C.c_int, [_P]),
    ("mcx_load", C.c_int, [_P, _P]),
    ("mcx_get", C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    ("mcx_put", C.c_int, [_P, C.c_int32, _P, C.c_size_t]),
    ("mcx_device_ptr", C.c_int, [_P, C.c_int32, C.POINTER(_P)]),
    ("mcx_state_save", C.c_int, [_P]),
    ("mcx_state_restore", C.c_int, [_P]),
    ("mcx_state_save_slot", C.c_int, [_P, C.c_int32]),
    ("mcx_state_restore_slot", C.c_int, [_P, C.c_int32]),
    ("mcx_opacity", C.c_int, [_P, C.POINTER(PhaseOpts), C.POINTER(PhaseStats)]),
    ("mcx_emission", C.c_int, [_P, C.POINTER(PhaseOpts), C.POINTER(PhaseStats)]),
    ("mcx_transport", C.c_int, [_P, C.POINTER(TransportOpts), C.POINTER(TransportStats)]),
    ("mcx_normalize_j", C.c_int, [_P]),
    ("mcx_balance", C.c_int, [_P, C.POINTER(BalanceOpts), C.POINTER(BalanceStats)]),
    ("mcx_iterate", C.c_int, [_P, C.POINTER(IterateOpts), C.POINTER(IterateStats)]),
    ("mcx_line_luminosities", C.c_int, [_P, C.POINTER(Lines)]),
    ("mcx_line_luminosities_nebula", C.c_int, [_P, C.c_int32, C.POINTER(Lines)]),
    ("mcx_batch_transport_ms", C.c_int, [_P, C.POINTER(C.c_double), C.c_int32]),
    ("mcx_line_sensitivities", C.c_int, [_P, C.POINTER(SensOpts), C.POINTER(SensOut)]),
    ("mcx_adjoint", C.c_int, [_P, C.POINTER(SensOpts), C.POINTER(AdjointOut)]),
    ("mcx_load_batched", C.c_int, [_P, _P, C.c_int32]),
    ("mcx_batch_info", C.c_int, [_P, C.POINTER(C.c_int32), _P]),
    ("mcx_transport_batched", C.c_int, [_P, C.POINTER(TransportOpts), C.POINTER(BatchPackets),
                                        C.POINTER(TransportStats)]),
    ("mcx_iterate_batched", C.c_int, [_P, C.POINTER(IterateOpts), C.POINTER(BatchPackets),
                                      C.POINTER(IterateStats)]),
    ("mcx_timer_start", C.c_int, [_P]),
    ("mcx_timer_stop", C.c_int, [_P, C.POINTER(C.c_float)]),
    ("mcx_version", C.c_char_p, []),
    ("mcx_transport_noalloc", C.c_int, [C.POINTER(NoallocTransportArgs), C.POINTER(TransportStats)]),
    ("mcx_noalloc_last_error", C.c_char_p, []),
]

_lib = None


def lib() -> C.CDLL:
    """The loaded libmcx.so; raises if it is missing (no fallback path exists)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        l = C.CDLL(str(LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(l, name)
            f.restype = res
            f.argtypes = args
        _lib = l
    return _lib


class McxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


def check_setup(rc: int) -> None:
    if rc != MCX_OK:
        raise McxError(rc, lib().mcx_setup_last_error().decode())


def as_ptr(a: np.ndarray) -> C.c_void_p:
    assert a.flags["C_CONTIGUOUS"]
    return C.c_void_p(a.ctypes.data)
