"""Thin Python handle over the C ABI (used by tests, bench and the serving loop).

Tracker.load(problem) uploads mesh, boundary conditions, nuclides,
materials, block map and source; Tracker.run(...) runs one batch of
histories on the GPU.  Every call checks the return code and raises
MCError with the library's message.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import (EIGEN_GEN_DTYPE, FISSION_SITE_DTYPE, MC_MODE_EVENT, MC_PREC_FP64, MC_TALLY_BATCH, MC_TALLY_SUM,
                   MC_TALLY_SUM_SQ, RAY_SEGMENT_DTYPE, SITE_DTYPE, TRACE_DTYPE, EigenDesc, Job, MCError, PersistDesc,
                   RunDesc, SourceDesc, Stats, TallyDesc, lib, ptr)
from .problems import Problem, Source, TallyDef


class Tracker:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib.mc_ctx_create(device, C.byref(h))
        if rc != 0:
            raise MCError(rc, f"mc_ctx_create(device={device}) failed (no usable CUDA device?)")
        self._h = h
        self.n_tet = 0

    # -- plumbing ---------------------------------------------------------
    def _ck(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = lib.mc_last_error(self._h)
            raise MCError(rc, f"{what}: {msg.decode() if msg else ''}")

    def close(self) -> None:
        if self._h:
            lib.mc_ctx_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- setup ------------------------------------------------------------
    def upload_mesh(self, xyz, tet_vtx, tet_block, tet_side_bid=None) -> None:
        xyz = np.ascontiguousarray(xyz, np.float64)
        tv = np.ascontiguousarray(tet_vtx, np.int32)
        blk = np.ascontiguousarray(tet_block, np.int32)
        bid = None if tet_side_bid is None else np.ascontiguousarray(tet_side_bid, np.int32)
        self._ck(lib.mc_mesh_upload(self._h, xyz.shape[0], ptr(xyz), tv.shape[0], ptr(tv), ptr(blk), ptr(bid)),
                 "mc_mesh_upload")
        self.n_tet = tv.shape[0]

    def set_bc(self, boundary_id: int, bc_type: int) -> None:
        self._ck(lib.mc_bc_set(self._h, boundary_id, bc_type), "mc_bc_set")

    def add_nuclide(self, E, sig_t, sig_s, awr) -> int:
        E, st, ss = (np.ascontiguousarray(a, np.float64) for a in (E, sig_t, sig_s))
        idx = C.c_int32()
        self._ck(lib.mc_nuclide_add(self._h, E.size, ptr(E), ptr(st), ptr(ss), float(awr), C.byref(idx)),
                 "mc_nuclide_add")
        return idx.value

    def set_fission(self, nuclide: int, nu_sig_f) -> None:
        """nu*sigma_f per grid point of a nuclide (None: not fissionable)."""
        f = None if nu_sig_f is None else np.ascontiguousarray(nu_sig_f, np.float64)
        self._ck(lib.mc_nuclide_set_fission(self._h, nuclide, ptr(f)), "mc_nuclide_set_fission")

    def add_material(self, material_id: int, nuclides, densities) -> None:
        n = np.ascontiguousarray(nuclides, np.int32)
        d = np.ascontiguousarray(densities, np.float64)
        self._ck(lib.mc_material_add(self._h, material_id, n.size, ptr(n), ptr(d)), "mc_material_add")

    def block_material_map(self, blocks, materials) -> None:
        b = np.ascontiguousarray(blocks, np.int32)
        m = np.ascontiguousarray(materials, np.int32)
        self._ck(lib.mc_block_material_map(self._h, b.size, ptr(b), ptr(m)), "mc_block_material_map")

    def set_hash_bins(self, n: int) -> None:
        self._ck(lib.mc_set_hash_bins(self._h, n), "mc_set_hash_bins")

    def set_source(self, s: Source) -> None:
        d = SourceDesc()
        d.space, d.energy = s.space, s.energy
        d.point[:] = s.point
        d.box_lo[:] = s.box_lo
        d.box_hi[:] = s.box_hi
        cyl = None
        if s.cyl_xy is not None:
            cyl = np.ascontiguousarray(s.cyl_xy, np.float64).reshape(-1)
            d.n_cyl = cyl.size // 2
            d.cyl_xy = cyl.ctypes.data_as(C.POINTER(C.c_double))
        d.cyl_r, d.cyl_z0, d.cyl_z1 = s.cyl_r, s.cyl_z0, s.cyl_z1
        d.watt_a, d.watt_b, d.mono_E = s.watt_a, s.watt_b, s.mono_E
        self._ck(lib.mc_source_set(self._h, C.byref(d)), "mc_source_set")

    def load(self, p: Problem) -> "Tracker":
        self.upload_mesh(p.xyz, p.tet_vtx, p.tet_block, p.tet_side_bid)
        for bid, t in p.bcs.items():
            self.set_bc(bid, t)
        for n in p.nuclides:
            k = self.add_nuclide(n.E, n.sig_t, n.sig_s, n.awr)
            if n.nu_sig_f is not None:
                self.set_fission(k, n.nu_sig_f)
        for m in p.materials:
            self.add_material(m.id, m.nuclides, m.densities)
        self.block_material_map(p.blocks, p.block_materials)
        self.set_hash_bins(p.hash_bins)
        self.set_source(p.source)
        if p.tally is not None:
            self.configure_tally(p.tally)
        self._ck(lib.mc_set_2d(self._h, 0 if p.z_2d is None else 1, 0.0 if p.z_2d is None else p.z_2d),
                 "mc_set_2d")
        return self

    def configure_tally(self, t: TallyDef) -> None:
        d = TallyDesc()
        d.estimator = t.estimator
        d.n_scores = len(t.scores)
        for j, s in enumerate(t.scores):
            d.scores[j] = s
        e = None if t.energy_edges is None else np.ascontiguousarray(t.energy_edges, np.float64)
        d.n_energy_bins = 0 if e is None else e.size - 1
        d.energy_edges = None if e is None else e.ctypes.data
        self._ck(lib.mc_tally_configure(self._h, C.byref(d)), "mc_tally_configure")

    def set_segment_limit(self, n: int) -> None:
        """Segments a history may walk before it ends as stuck (0: the mesh-size default)."""
        self._ck(lib.mc_set_segment_limit(self._h, n), "mc_set_segment_limit")

    def segment_limit(self) -> int:
        v = C.c_int64()
        self._ck(lib.mc_segment_limit(self._h, C.byref(v)), "mc_segment_limit")
        return v.value

    def enable_rays(self, n_rays: int, max_segments: int = 4096) -> None:
        """Record every segment of the first n_rays histories of each run (0: off)."""
        self._ck(lib.mc_rays_enable(self._h, n_rays, max_segments), "mc_rays_enable")

    def rays(self) -> np.ndarray:
        """Segments recorded by the last run (RAY_SEGMENT_DTYPE), ray by ray."""
        n = C.c_int64()
        lib.mc_rays_download(self._h, None, 0, C.byref(n))
        out = np.zeros(n.value, RAY_SEGMENT_DTYPE)
        self._ck(lib.mc_rays_download(self._h, ptr(out), out.size, C.byref(n)), "mc_rays_download")
        return out

    def tally_size(self) -> int:
        n = C.c_int64()
        self._ck(lib.mc_tally_size(self._h, C.byref(n)), "mc_tally_size")
        return n.value

    # -- run --------------------------------------------------------------
    def run(self, n: int, first: int = 0, seed: int = 1, mode: int = MC_MODE_EVENT,
            precision: int = MC_PREC_FP64, bank_size: int = 0, block_size: int = 0,
            max_seg: int = 0, traces: bool = False, accumulate: bool = False,
            sort_queue: bool = False, profile: bool = False, sites: np.ndarray | None = None,
            refill: bool = False, batch_sizes=None, graph: bool = False, tail: int = 0,
            batch_results=None, walk_blocks: int = 0) -> Stats:
        """One batch of n histories, or, with batch_sizes (adding up to n),
        consecutive batches run through one pipeline (needs accumulate).
        batch_results: one float64 array of tally_size() per batch, each
        receiving the SUM tally as it stands once its batch is folded in.
        walk_blocks: the FP64 walk kernel's build, 5 or 4 resident blocks of
        128 threads per SM (0: 5); results are the same, speed depends on the
        problem (autotune tries both)."""
        if sites is not None:
            assert sites.dtype == SITE_DTYPE and sites.size >= n and sites.flags["C_CONTIGUOUS"]
        bs = None if batch_sizes is None else np.ascontiguousarray(batch_sizes, np.int64)
        outs = None
        if batch_results is not None:
            nbat = 1 if bs is None else bs.size
            assert len(batch_results) == nbat
            for r in batch_results:
                assert r.dtype == np.float64 and r.flags["C_CONTIGUOUS"] and r.size == self.tally_size()
            outs = (C.c_void_p * nbat)(*[r.ctypes.data for r in batch_results])
        d = RunDesc(first, n, bank_size, seed, precision, mode, block_size, max_seg, int(traces),
                    int(accumulate), int(sort_queue), int(profile), int(refill), 0 if bs is None else bs.size,
                    int(graph), int(tail), None if sites is None else sites.ctypes.data,
                    None if bs is None else bs.ctypes.data,
                    None if outs is None else C.cast(outs, C.c_void_p), int(walk_blocks))
        self._ck(lib.mc_run(self._h, C.byref(d)), "mc_run")
        return self.stats()

    def eigen(self, n: int, generations: int, inactive: int = 0, seed: int = 1, precision: int = MC_PREC_FP64,
              mode: int = MC_MODE_EVENT, bank_size: int = 0, block_size: int = 0, max_seg: int = 0,
              sort_queue: int = 0, graph: bool = False, keff0: float = 0.0, watt=(0.0, 0.0), capacity: int = 0,
              initial_source: np.ndarray | None = None, tail: int = 0) -> np.ndarray:
        """k-eigenvalue generations of n histories; returns one
        EIGEN_GEN_DTYPE record per generation."""
        if initial_source is not None:
            assert initial_source.dtype == SITE_DTYPE and initial_source.size == n
            initial_source = np.ascontiguousarray(initial_source)
        d = EigenDesc(n, generations, inactive, seed, precision, mode, bank_size, block_size, max_seg,
                      int(sort_queue), int(graph), int(tail), keff0, watt[0], watt[1], capacity,
                      None if initial_source is None else initial_source.ctypes.data)
        out = np.zeros(generations, EIGEN_GEN_DTYPE)
        self._ck(lib.mc_eigen_run(self._h, C.byref(d), ptr(out)), "mc_eigen_run")
        return out

    def eigen_source(self, n: int) -> np.ndarray:
        """Source sites of the next generation after the last eigen run."""
        out = np.zeros(n, SITE_DTYPE)
        self._ck(lib.mc_eigen_source_download(self._h, ptr(out), n), "mc_eigen_source_download")
        return out

    def fission_bank(self) -> np.ndarray:
        """The last generation's fission bank in (parent, progeny) order."""
        m = C.c_int64()
        self._ck(lib.mc_eigen_fission_bank_download(self._h, None, 0, C.byref(m)), "mc_eigen_fission_bank_download")
        out = np.zeros(m.value, FISSION_SITE_DTYPE)
        self._ck(lib.mc_eigen_fission_bank_download(self._h, ptr(out), out.size, C.byref(m)),
                 "mc_eigen_fission_bank_download")
        return out

    def autotune(self, trial: int = 200_000, **base) -> tuple[dict, float]:
        """Best event-form parameters on trial batches; returns (params, histories/s)."""
        d = RunDesc(base.get("first", 0), trial, base.get("bank_size", 0), base.get("seed", 1),
                    base.get("precision", MC_PREC_FP64), MC_MODE_EVENT, base.get("block_size", 0),
                    base.get("max_seg", 0), 0, 0, base.get("sort_queue", 0), 0, base.get("refill", 0), 0,
                    base.get("graph", 0), 0, None, None, None, base.get("walk_blocks", 0))
        out = RunDesc()
        rate = C.c_double()
        self._ck(lib.mc_autotune(self._h, C.byref(d), trial, C.byref(out), C.byref(rate)), "mc_autotune")
        return ({"bank_size": out.bank_size, "block_size": out.block_size, "max_seg": out.max_seg_per_advance,
                 "sort_queue": out.sort_queue, "refill": bool(out.refill), "graph": bool(out.graph),
                 "walk_blocks": out.walk_blocks},
                rate.value)

    def sample_sites(self, n: int, first: int = 0, seed: int = 1, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros(n, SITE_DTYPE)
        self._ck(lib.mc_source_sample(self._h, first, n, seed, ptr(out)), "mc_source_sample")
        return out

    def set_stream(self, stream_handle: int | None) -> None:
        self._ck(lib.mc_ctx_set_stream(self._h, stream_handle), "mc_ctx_set_stream")

    def sync(self) -> None:
        self._ck(lib.mc_sync(self._h), "mc_sync")

    def stats(self) -> Stats:
        s = Stats()
        self._ck(lib.mc_stats_get(self._h, C.byref(s)), "mc_stats_get")
        return s

    def tally(self, kind: int = MC_TALLY_BATCH, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.zeros(self.tally_size(), np.float64)
        self._ck(lib.mc_tally_download(self._h, kind, ptr(out), out.size), "mc_tally_download")
        return out

    def tally_sum(self) -> np.ndarray:
        return self.tally(MC_TALLY_SUM)

    def tally_sum_sq(self) -> np.ndarray:
        return self.tally(MC_TALLY_SUM_SQ)

    def reset_tally(self) -> None:
        self._ck(lib.mc_tally_reset(self._h), "mc_tally_reset")

    def traces(self, n: int) -> np.ndarray:
        out = np.zeros(n, TRACE_DTYPE)
        self._ck(lib.mc_trace_download(self._h, ptr(out), n), "mc_trace_download")
        return out

    def batches_done(self) -> int:
        v = C.c_int64()
        self._ck(lib.mc_batches_done(self._h, C.byref(v)), "mc_batches_done")
        return v.value


def run_persistent(jobs, precision: int = MC_PREC_FP64, slots: int = 0, block_size: int = 0,
                   traces: bool = False, wait_limit: int = 0):
    """mc_run_persistent: jobs is a list of (tracker, first_history,
    n_histories, seed), one batch each, in the order their histories are
    numbered; every batch folds into its tracker's SUM/SUM_SQ.  Returns
    (Stats, traces of the run's histories in job order or None)."""
    arr = (Job * len(jobs))()
    total = 0
    for i, (t, first, n, seed) in enumerate(jobs):
        arr[i] = Job(t._h.value if isinstance(t._h, C.c_void_p) else t._h, first, n, seed)
        total += n
    tr = np.zeros(total, TRACE_DTYPE) if traces else None
    d = PersistDesc(precision, block_size, slots, int(traces), wait_limit, None if tr is None else tr.ctypes.data)
    st = Stats()
    rc = lib.mc_run_persistent(C.byref(d), len(jobs), arr, C.byref(st))
    if rc != 0:
        msg = lib.mc_last_error(jobs[0][0]._h)
        raise MCError(rc, f"mc_run_persistent: {msg.decode() if msg else ''}")
    return st, tr
