"""Host-side Python mirror of the reference's set-up and iteration phases,
calling libmcx.so through its C ABI.

``Setup`` is the model built from an input deck (readInput / initCartesianGrid
/ initXSecArray / setContinuum / fillGrid of the reference).  ``Context`` holds
the device-resident copy and runs the phases of one MC iteration the way
iterateMC (source/iteration_mod.f90:32-1497) sequences them.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

from . import abi
from .abi import lib


class Setup:
    def __init__(self, input_file: str | Path, data_dir: str | Path, mesh_mode: int = abi.MESH_REFERENCE):
        opts = abi.SetupOpts(mesh_mode=mesh_mode)
        h = C.c_void_p()
        abi.check_setup(lib().mcx_setup_from_input(str(input_file).encode(), str(data_dir).encode(),
                                                   C.byref(opts), C.byref(h)))
        self._h = h
        info = abi.SetupInfo()
        abi.check_setup(lib().mcx_setup_info_get(h, C.byref(info)))
        self.info = info

    def close(self) -> None:
        if self._h:
            lib().mcx_setup_free(self._h)
            self._h = None

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    # sizes
    @property
    def n_cells(self) -> int:
        return self.info.n_cells

    @property
    def nbins(self) -> int:
        return self.info.nbins

    _DT = {abi.ARR_ACTIVE: np.int32, **{k: np.int32 for k in abi.INT_SARR}, **{k: np.float64 for k in abi.F64_SARR}}

    def get(self, arr_id: int) -> np.ndarray:
        n = C.c_int64()
        abi.check_setup(lib().mcx_setup_len(self._h, arr_id, C.byref(n)))
        a = np.empty(n.value, dtype=self._DT.get(arr_id, np.float32))
        abi.check_setup(lib().mcx_setup_get(self._h, arr_id, abi.as_ptr(a), a.nbytes))
        return a

    def set(self, arr_id: int, a: np.ndarray) -> None:
        a = np.ascontiguousarray(a, dtype=self._DT.get(arr_id, np.float32))
        abi.check_setup(lib().mcx_setup_set(self._h, arr_id, abi.as_ptr(a), a.nbytes))


class Context:
    """One device context (libmcx's mcx_ctx) holding one loaded model."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib().mcx_ctx_create(device, C.byref(h))
        if rc != abi.MCX_OK:
            raise abi.McxError(rc, lib().mcx_setup_last_error().decode())
        self._h = h
        self.setup: Setup | None = None
        self.batch: list[Setup] | None = None
        self.cell_offsets: np.ndarray | None = None
        self._cells = 0

    def close(self) -> None:
        if self._h:
            lib().mcx_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc: int) -> None:
        if rc != abi.MCX_OK:
            buf = C.create_string_buffer(1024)
            lib().mcx_last_error(self._h, buf, 1024)
            raise abi.McxError(rc, buf.value.decode())

    def load(self, setup: Setup) -> None:
        self._check(lib().mcx_load(self._h, setup.handle))
        self.setup = setup
        self.batch = None
        self.cell_offsets = None
        self._cells = setup.info.n_cells

    def load_batched(self, setups: list[Setup]) -> None:
        """A batch of nebulae in one context (mcx_load_batched): per-cell arrays are the concatenation
        of the nebulae's behind one dump cell; `cell_offsets[b]` is nebula b's offset."""
        arr = (C.c_void_p * len(setups))(*[x.handle.value for x in setups])
        self._check(lib().mcx_load_batched(self._h, arr, len(setups)))
        n = C.c_int32()
        offs = (C.c_int32 * (len(setups) + 1))()
        self._check(lib().mcx_batch_info(self._h, C.byref(n), offs))
        self.setup = setups[0]
        self.batch = list(setups)
        self.cell_offsets = np.array(offs[:], dtype=np.int64)
        self._cells = int(self.cell_offsets[-1])

    def nebula_cells(self, a: np.ndarray, b: int) -> np.ndarray:
        """The cells 1..nCells of nebula b from a batch-wide per-cell array (cells on the last axis)."""
        return a[..., self.cell_offsets[b] + 1:self.cell_offsets[b + 1] + 1]

    def _batch_packets(self, n_packets, seeds, counter_bases, n_photons_norm):
        nb = len(self.batch)
        keep = dict(n=np.ascontiguousarray(np.broadcast_to(np.asarray(n_packets, dtype=np.int64), (nb,))),
                    s=np.ascontiguousarray(np.broadcast_to(np.asarray(seeds, dtype=np.uint64), (nb,))),
                    c=np.ascontiguousarray(np.broadcast_to(np.asarray(0 if counter_bases is None else counter_bases,
                                                                      dtype=np.uint64), (nb,))))
        if n_photons_norm is not None:
            keep["p"] = np.ascontiguousarray(np.broadcast_to(np.asarray(n_photons_norm, dtype=np.int64), (nb,)))
        pk = abi.BatchPackets(n_packets=keep["n"].ctypes.data, seed=keep["s"].ctypes.data,
                              counter_base=keep["c"].ctypes.data,
                              n_photons_norm=keep["p"].ctypes.data if "p" in keep else None)
        return pk, keep

    def transport_batched(self, n_packets, seeds, counter_bases=None, precision: int = abi.PREC_FP32_GEOM,
                          zero: bool = True, n_photons_norm=None, block_size: int = 0,
                          grid_mult: int = 0, emit_batch: int = 0) -> abi.TransportStats:
        """Every nebula's packets in one launch: n_packets, seeds, counter_bases per nebula (scalars broadcast)."""
        pk, keep = self._batch_packets(n_packets, seeds, counter_bases, n_photons_norm)
        o = abi.TransportOpts(istar=1, precision=precision, zero_estimators=1 if zero else 0, block_size=block_size,
                              grid_mult=grid_mult, emit_batch=emit_batch)
        st = abi.TransportStats()
        self._check(lib().mcx_transport_batched(self._h, C.byref(o), C.byref(pk), C.byref(st)))
        return st

    def iterate_batched(self, n_packets, seeds, counter_bases=None, n_iterate_mc: int = 1,
                        transport_precision: int = abi.PREC_FP32_GEOM, balance_precision: int = abi.BAL_MIXED,
                        emission_precision: int = abi.PHASE_MIXED, launch: dict | None = None) -> abi.IterateStats:
        """One MC iteration of every nebula of the batch in one ABI call; `launch` = the transport's
        block_size / grid_mult / emit_batch (e.g. from autotune.tune_transport), library defaults if None."""
        pk, keep = self._batch_packets(n_packets, seeds, counter_bases, None)
        L = launch or {}
        o = abi.IterateOpts(n_iterate_mc=n_iterate_mc, transport_precision=transport_precision,
                            balance_precision=balance_precision, emission_precision=emission_precision,
                            transport_block_size=L.get("block_size", 0), transport_grid_mult=L.get("grid_mult", 0),
                            transport_emit_batch=L.get("emit_batch", 0))
        st = abi.IterateStats()
        self._check(lib().mcx_iterate_batched(self._h, C.byref(o), C.byref(pk), C.byref(st)))
        return st

    def batch_transport_ms(self) -> np.ndarray:
        """When each nebula's last packet of the latest batched transport finished, ms after its launch began."""
        out = np.zeros(len(self.cell_offsets) - 1, dtype=np.float64)
        self._check(lib().mcx_batch_transport_ms(self._h, out.ctypes.data_as(C.POINTER(C.c_double)), out.size))
        return out

    def _shape(self, arr_id: int) -> tuple[tuple, type]:
        s = self.setup.info
        C1, nb = self._cells + 1, s.nbins
        f32, f64 = np.float32, np.float64
        shapes = {
            abi.ARR_OPACITY: ((nb, C1), f32), abi.ARR_RECPDF: ((nb, C1), f32), abi.ARR_SCAOPAC: ((nb, C1), f32),
            abi.ARR_DUSTPDF: ((nb, C1), f32), abi.ARR_JSTE: ((nb, C1), f64), abi.ARR_H_EST: ((nb, C1), f64),
            abi.ARR_ESCAPED: (((nb + 1, C1) if s.n_angle_bins == 0 else (s.n_angle_bins + 1, nb + 1, C1)), f64), abi.ARR_TOTAL_LINES: ((C1,), f32), abi.ARR_HDEN: ((C1,), f32),
            abi.ARR_TE: ((C1,), f32), abi.ARR_NE: ((C1,), f32), abi.ARR_TEOLD: ((C1,), f32),
            abi.ARR_NEOLD: ((C1,), f32), abi.ARR_VOLUME: ((C1,), f32), abi.ARR_GAUNT_TE: ((C1,), f32),
            abi.ARR_NDUST: ((C1,), f32), abi.ARR_LG_CONVERGED: ((C1,), np.int32),
            abi.ARR_LG_BLACK: ((C1,), np.int32), abi.ARR_N_ITER_T: ((C1,), np.int32), abi.ARR_FOR_LINES: ((C1,), f32),
            abi.ARR_IONDEN: ((s.nstages, max(s.n_elem_used, 1), C1), f32),
            abi.ARR_TDUST: ((self._dust_planes(), C1), f32),
            abi.ARR_BAL_RESID: ((C1,), np.float64),
        }
        return shapes[arr_id]

    def _dust_planes(self) -> int:
        if not self.setup.info.lg_dust:
            return 0
        d = self.setup.get(abi.SARR_DUST_DIMS)
        return int((d[0] + 1) * (d[1] + 1))

    def get(self, arr_id: int) -> np.ndarray:
        shape, dt = self._shape(arr_id)
        a = np.empty(shape, dtype=dt)
        self._check(lib().mcx_get(self._h, arr_id, abi.as_ptr(a), a.nbytes))
        return a

    def put(self, arr_id: int, a: np.ndarray) -> None:
        shape, dt = self._shape(arr_id)
        a = np.ascontiguousarray(a, dtype=dt).reshape(shape)
        self._check(lib().mcx_put(self._h, arr_id, abi.as_ptr(a), a.nbytes))

    def opacity(self, n_iterate_mc: int = 1) -> abi.PhaseStats:
        st = abi.PhaseStats()
        o = abi.PhaseOpts(n_iterate_mc=n_iterate_mc)
        self._check(lib().mcx_opacity(self._h, C.byref(o), C.byref(st)))
        return st

    def emission(self, n_iterate_mc: int = 1, precision: int = abi.PHASE_EXACT) -> abi.PhaseStats:
        st = abi.PhaseStats()
        o = abi.PhaseOpts(n_iterate_mc=n_iterate_mc, precision=precision)
        self._check(lib().mcx_emission(self._h, C.byref(o), C.byref(st)))
        return st

    def transport(self, n_packets: int, seed: int = 0, counter_base: int = 0, precision: int = abi.PREC_FP32_GEOM,
                  zero: bool = True, n_photons_norm: int = 0, block_size: int = 0, grid_mult: int = 0,
                  emit_batch: int = 0, handoff_emissions: int = 0, istar: int = 1) -> abi.TransportStats:
        """Packets of ionising source `istar` (1-based).  handoff_emissions:
        re-emissions after which a history moves to the trapped-packet kernel
        (0 = library default, -1 = never); it changes only where a history
        runs, never its result."""
        o = abi.TransportOpts(istar=istar, precision=precision, n_packets=n_packets, seed=seed, counter_base=counter_base,
                              n_photons_norm=n_photons_norm, zero_estimators=1 if zero else 0,
                              block_size=block_size, grid_mult=grid_mult, emit_batch=emit_batch,
                              handoff_emissions=handoff_emissions)
        st = abi.TransportStats()
        self._check(lib().mcx_transport(self._h, C.byref(o), C.byref(st)))
        return st

    def balance(self, max_rounds: int = 0, precision: int = abi.BAL_FP64,
                atom_solves: bool = False, converge: bool = False, fix_te: bool = False) -> abi.BalanceStats:
        """updateCell for every cell (Te, Ne, ionDen, lgConverged) from the normalised J.  atom_solves
        (mixed precision): solve every ion's levels per cell instead of reading the cooling surfaces;
        converge: converge every cell tightly instead of iterateT's stopping rules; fix_te (with
        converge): hold every cell's Te, converge its ladder there and leave heating - cooling in
        ARR_BAL_RESID."""
        o = abi.BalanceOpts(precision=precision, max_rounds=max_rounds, atom_solves=int(atom_solves),
                            converge=int(converge), fix_te=int(fix_te))
        st = abi.BalanceStats()
        self._check(lib().mcx_balance(self._h, C.byref(o), C.byref(st)))
        return st

    def iterate(self, n_packets: int, n_iterate_mc: int = 1, seed: int = 0, counter_base: int = 0,
                transport_precision: int = abi.PREC_FP32_GEOM, balance_precision: int = abi.BAL_MIXED,
                emission_precision: int = abi.PHASE_MIXED) -> abi.IterateStats:
        """One MC iteration (opacity, emission, transport, normalisation, balance) in one ABI call."""
        o = abi.IterateOpts(n_iterate_mc=n_iterate_mc, transport_precision=transport_precision,
                            balance_precision=balance_precision, emission_precision=emission_precision,
                            n_packets=n_packets, seed=seed, counter_base=counter_base)
        st = abi.IterateStats()
        self._check(lib().mcx_iterate(self._h, C.byref(o), C.byref(st)))
        return st

    def line_luminosities(self, nebula: int | None = None) -> dict:
        """outputGas's analytical line luminosities and ionic volume averages from the current state
        (source/output_mod.f90:13-805); of nebula `nebula` for a batch.

        Returns hbeta_vol [1e36 erg/s] (x8 in symmetricXYZ mode), relative (line sums divided by
        HbetaVol), n_cells, kernel_ms, hydro[30,14,8] at [iz-1, iup-2, ilow-1], hei[34],
        forb and wav [30, nstages, 30, 30] at [elem-1, ion-1, i-1, j-1] (i lower, j upper level),
        te_vol and ion_vol [30, nstages] at [elem-1, ion-1]."""
        S = self.setup.info.nstages
        hydro = np.zeros(30 * 14 * 8)
        hei = np.zeros(34)
        forb = np.zeros(30 * S * 30 * 30)
        wav = np.zeros(30 * S * 30 * 30)
        te_vol = np.zeros(30 * S)
        ion_vol = np.zeros(30 * S)
        o = abi.Lines(hydro_vol=hydro.ctypes.data, hei_vol=hei.ctypes.data, forb_vol=forb.ctypes.data,
                      wav=wav.ctypes.data, te_vol=te_vol.ctypes.data, ion_vol=ion_vol.ctypes.data)
        if nebula is None:
            self._check(lib().mcx_line_luminosities(self._h, C.byref(o)))
        else:
            self._check(lib().mcx_line_luminosities_nebula(self._h, nebula, C.byref(o)))
        # the ABI arrays are column-major (the reference's layouts): reverse the axes
        return dict(hbeta_vol=o.hbeta_vol, relative=bool(o.relative), n_cells=int(o.n_cells),
                    kernel_ms=float(o.kernel_ms),
                    hydro=hydro.reshape(8, 14, 30).transpose(2, 1, 0).copy(),
                    hei=hei, forb=forb.reshape(30, 30, S, 30).transpose(3, 2, 1, 0).copy(),
                    wav=wav.reshape(30, 30, S, 30).transpose(3, 2, 1, 0).copy(),
                    te_vol=te_vol.reshape(S, 30).T.copy(), ion_vol=ion_vol.reshape(S, 30).T.copy())

    def line_sensitivities(self, lines, abun_z=(), h: float = 1e-3, precision: int = abi.BAL_MIXED,
                           per_cell: bool = True, reference_stopping: bool = False) -> dict:
        """Frozen-field sensitivities (mcx_line_sensitivities): with the context's J fixed, the outputGas
        volume sums L of the forbidden lines `lines` [(elem, ion, lower, upper), ...], dL/dHden per cell
        ([n_lines, nCells+1]) and dL/d(elemAbun) of the elements `abun_z` ([n_lines, len(abun_z)]),
        by forward differences of relative step h of tightly converged balances (of balances stopped
        by iterateT's own rules with reference_stopping)."""
        n = len(lines)
        refs = (abi.LineRef * n)(*[abi.LineRef(*map(int, l)) for l in lines])
        z = np.ascontiguousarray(np.asarray(abun_z, dtype=np.int32))
        L = np.zeros(n)
        dh = np.zeros((n, self._cells + 1)) if per_cell else None
        da = np.zeros((n, max(len(z), 1)))
        o = abi.SensOpts(n_lines=n, n_abun=len(z), lines=C.cast(refs, C.c_void_p),
                         abun_z=z.ctypes.data if len(z) else None, h=h, precision=precision,
                         reference_stopping=int(reference_stopping))
        out = abi.SensOut(L=L.ctypes.data, dL_dhden=dh.ctypes.data if per_cell else None,
                          dL_dabun=da.ctypes.data if len(z) else None)
        self._check(lib().mcx_line_sensitivities(self._h, C.byref(o), C.byref(out)))
        return dict(L=L, dL_dhden=dh, dL_dabun=da[:, :len(z)], kernel_ms=float(out.kernel_ms),
                    branch_cells_hden=int(out.branch_cells_hden), branch_cells_abun=int(out.branch_cells_abun))

    def adjoint(self, lines, abun_z=(), h: float = 1e-3, precision: int = abi.BAL_MIXED,
                per_cell: bool = True) -> dict:
        """The implicit-function adjoint of the converged balance at the context's J (mcx_adjoint): the
        outputGas volume sums L of the forbidden lines `lines` [(elem, ion, lower, upper), ...] after a
        tightly converged balance, dL/dHden per cell ([n_lines, nCells+1]), dTe/dHden of each cell's root
        ([nCells+1]) and dL/d(elemAbun) of the elements `abun_z` ([n_lines, len(abun_z)]), from central
        differences (relative step h) of evaluations with every Te held."""
        n = len(lines)
        refs = (abi.LineRef * n)(*[abi.LineRef(*map(int, l)) for l in lines])
        z = np.ascontiguousarray(np.asarray(abun_z, dtype=np.int32))
        L = np.zeros(n)
        dh = np.zeros((n, self._cells + 1)) if per_cell else None
        dt = np.zeros(self._cells + 1) if per_cell else None
        da = np.zeros((n, max(len(z), 1)))
        o = abi.SensOpts(n_lines=n, n_abun=len(z), lines=C.cast(refs, C.c_void_p),
                         abun_z=z.ctypes.data if len(z) else None, h=h, precision=precision)
        out = abi.AdjointOut(L=L.ctypes.data, dL_dhden=dh.ctypes.data if per_cell else None,
                             dL_dabun=da.ctypes.data if len(z) else None,
                             dte_dhden=dt.ctypes.data if per_cell else None)
        self._check(lib().mcx_adjoint(self._h, C.byref(o), C.byref(out)))
        return dict(L=L, dL_dhden=dh, dte_dhden=dt, dL_dabun=da[:, :len(z)], kernel_ms=float(out.kernel_ms),
                    pinned_cells=int(out.pinned_cells), no_solution_cells=int(out.no_solution_cells))

    def state_save(self, slot: int = 0) -> None:
        """Device-side snapshot, in slot `slot`, of everything an iteration
        hands to the next (gas state, the skip rule's kept opacity and
        emission CDF, Gaunt-cache temperatures, grain arrays)."""
        self._check(lib().mcx_state_save_slot(self._h, slot))

    def state_restore(self, slot: int = 0) -> None:
        self._check(lib().mcx_state_restore_slot(self._h, slot))

    def normalize_j(self) -> None:
        self._check(lib().mcx_normalize_j(self._h))

    def sync(self) -> None:
        self._check(lib().mcx_sync(self._h))

    def timer_start(self) -> None:
        self._check(lib().mcx_timer_start(self._h))

    def timer_stop(self) -> float:
        ms = C.c_float()
        self._check(lib().mcx_timer_stop(self._h, C.byref(ms)))
        return ms.value
