"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use
this module, as the checker and the timed CPU baseline; the product never
imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

from . import build as _build

_I32, _I64, _U64, _D, _P = C.c_int32, C.c_int64, C.c_uint64, C.c_double, C.c_void_p


class OracleSource(C.Structure):
    _fields_ = [("space", C.c_int32), ("energy", C.c_int32),
                ("point", C.c_double * 3), ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3),
                ("n_cyl", C.c_int32), ("pad", C.c_int32), ("cyl_xy", C.POINTER(C.c_double)),
                ("cyl_r", C.c_double), ("cyl_z0", C.c_double), ("cyl_z1", C.c_double),
                ("watt_a", C.c_double), ("watt_b", C.c_double), ("mono_E", C.c_double)]


class OracleStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("n_hist", "n_seg", "n_coll", "n_leak", "n_absorb", "n_cutoff",
                                        "n_stuck", "n_lost", "n_badxs")] + [("leak_weight", C.c_double)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


TRACE_DTYPE = np.dtype([("id", "<i8"), ("hash", "<u8"), ("status", "<i4"), ("n_seg", "<i4"),
                        ("n_coll", "<i4"), ("elem", "<i4"), ("face", "<i4"), ("pad", "<i4"),
                        ("E", "<f8"), ("x", "<f8"), ("y", "<f8"), ("z", "<f8")])

FSITE_DTYPE = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("u", "<f8"), ("v", "<f8"), ("w", "<f8"),
                        ("E", "<f8"), ("wgt", "<f8"), ("parent", "<i8"), ("progeny", "<i4"), ("pad", "<i4")])
RAY_DTYPE = np.dtype([("id", "<i8"), ("segment", "<i4"), ("intersections", "<i4"), ("elem", "<i4"),
                      ("pad", "<i4"), ("start", "<f8", (3,)), ("end", "<f8", (3,)), ("E", "<f8"),
                      ("wgt", "<f8"), ("seed_tracking", "<u8")])
GEN_DTYPE = np.dtype([("k_generation", "<f8"), ("k_collision", "<f8"), ("k_absorption", "<f8"), ("keff", "<f8"),
                      ("keff_std", "<f8"), ("leakage", "<f8"), ("n_sites", "<i8"), ("n_seg", "<i8"),
                      ("n_coll", "<i8")])

_SIG = {
    "oracle_create": ([], _P),
    "oracle_destroy": ([_P], None),
    "oracle_error": ([_P], C.c_char_p),
    "oracle_set_mesh": ([_P, _I64, _P, _I64, _P, _P, _P], C.c_int),
    "oracle_set_bc": ([_P, _I32, _I32], C.c_int),
    "oracle_add_nuclide": ([_P, _I64, _P, _P, _P, _D], C.c_int),
    "oracle_add_material": ([_P, _I32, _I32, _P, _P], C.c_int),
    "oracle_block_map": ([_P, _I32, _P, _P], C.c_int),
    "oracle_set_source": ([_P, C.POINTER(OracleSource)], C.c_int),
    "oracle_set_hash_bins": ([_P, _I32], C.c_int),
    "oracle_set_tally": ([C.c_void_p, C.c_int32, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p], C.c_int),
    "oracle_tally_size": ([C.c_void_p], C.c_int64),
    "oracle_set_2d": ([C.c_void_p, C.c_int32, C.c_double], C.c_int),
    "oracle_run": ([_P, _I64, _I64, _U64, C.c_int, _P, _P, C.POINTER(OracleStats)], C.c_int),
    "oracle_run_sites": ([_P, _I64, _I64, _U64, _P, C.c_int, _P, _P, C.POINTER(OracleStats)], C.c_int),
    "oracle_set_segment_limit": ([_P, _I64], C.c_int),
    "oracle_segment_limit": ([_P], _I64),
    "oracle_rays_enable": ([_P, _I32, _I32], C.c_int),
    "oracle_rays": ([_P, _P, _I64, C.POINTER(_I64)], C.c_int),
    "oracle_set_fission": ([_P, _I32, _P], C.c_int),
    "oracle_eigen_run": ([_P, _I64, _I32, _I32, _U64, _D, _D, _D, _I64, C.c_int, _P, _P, _P, _P, _I64, _P, _P],
                         C.c_int),
    "oracle_log": ([_D], _D),
    "oracle_quotient": ([_D, _D], _D),
    "oracle_prn": ([C.POINTER(_U64)], _D),
    "oracle_future_seed": ([_U64, _U64], _U64),
    "oracle_init_seed": ([_I64, _U64, C.c_int], _U64),
    "oracle_xs_index": ([_P, _I32, _D, C.POINTER(_D)], C.c_int),
    "oracle_macro_xs": ([_P, _I32, _D, C.POINTER(_D)], C.c_int),
    "oracle_mesh_info": ([_P, C.POINTER(_P), C.POINTER(_P)], C.c_int),
    "oracle_locate": ([_P, _P, _P], C.c_int),
}


def _load() -> C.CDLL:
    lib = C.CDLL(str(_build.build()))
    for name, (args, res) in _SIG.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    return lib


lib = _load()


def _p(a):
    return None if a is None else C.c_void_p(a.ctypes.data)


class Oracle:
    """CPU restatement loaded with one problem (a macaw_gb300.problems.Problem)."""

    def __init__(self, problem=None):
        self.h = lib.oracle_create()
        self.n_tet = 0
        self._keep = []
        if problem is not None:
            self.load(problem)

    def __del__(self):
        try:
            if self.h:
                lib.oracle_destroy(self.h)
                self.h = None
        except Exception:
            pass

    def _ck(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"{what}: {lib.oracle_error(self.h).decode()}")

    def load(self, p) -> "Oracle":
        xyz = np.ascontiguousarray(p.xyz, np.float64)
        tv = np.ascontiguousarray(p.tet_vtx, np.int32)
        blk = np.ascontiguousarray(p.tet_block, np.int32)
        bid = np.ascontiguousarray(p.tet_side_bid, np.int32)
        self._ck(lib.oracle_set_mesh(self.h, xyz.shape[0], _p(xyz), tv.shape[0], _p(tv), _p(blk), _p(bid)),
                 "oracle_set_mesh")
        self.n_tet = tv.shape[0]
        for b, t in p.bcs.items():
            self._ck(lib.oracle_set_bc(self.h, b, t), "oracle_set_bc")
        for k, n in enumerate(p.nuclides):
            E, st, ss = (np.ascontiguousarray(a, np.float64) for a in (n.E, n.sig_t, n.sig_s))
            self._ck(lib.oracle_add_nuclide(self.h, E.size, _p(E), _p(st), _p(ss), n.awr), "oracle_add_nuclide")
            if getattr(n, "nu_sig_f", None) is not None:
                f = np.ascontiguousarray(n.nu_sig_f, np.float64)
                self._ck(lib.oracle_set_fission(self.h, k, _p(f)), "oracle_set_fission")
        for m in p.materials:
            ni = np.ascontiguousarray(m.nuclides, np.int32)
            d = np.ascontiguousarray(m.densities, np.float64)
            self._ck(lib.oracle_add_material(self.h, m.id, ni.size, _p(ni), _p(d)), "oracle_add_material")
        b = np.ascontiguousarray(p.blocks, np.int32)
        mm = np.ascontiguousarray(p.block_materials, np.int32)
        self._ck(lib.oracle_block_map(self.h, b.size, _p(b), _p(mm)), "oracle_block_map")
        self._ck(lib.oracle_set_hash_bins(self.h, p.hash_bins), "oracle_set_hash_bins")
        s = p.source
        d = OracleSource()
        d.space, d.energy = s.space, s.energy
        d.point[:] = s.point
        d.box_lo[:] = s.box_lo
        d.box_hi[:] = s.box_hi
        if s.cyl_xy is not None:
            cyl = np.ascontiguousarray(s.cyl_xy, np.float64).reshape(-1)
            self._keep.append(cyl)
            d.n_cyl = cyl.size // 2
            d.cyl_xy = cyl.ctypes.data_as(C.POINTER(C.c_double))
        d.cyl_r, d.cyl_z0, d.cyl_z1 = s.cyl_r, s.cyl_z0, s.cyl_z1
        d.watt_a, d.watt_b, d.mono_E = s.watt_a, s.watt_b, s.mono_E
        self._ck(lib.oracle_set_source(self.h, C.byref(d)), "oracle_set_source")
        if getattr(p, "tally", None) is not None:
            self.set_tally(p.tally)
        if getattr(p, "z_2d", None) is not None:
            lib.oracle_set_2d(self.h, 1, p.z_2d)
        return self

    def set_tally(self, t) -> None:
        """t: macaw_gb300.problems.TallyDef."""
        sc = np.ascontiguousarray(t.scores, np.int32)
        e = None if t.energy_edges is None else np.ascontiguousarray(t.energy_edges, np.float64)
        self._ck(lib.oracle_set_tally(self.h, t.estimator, sc.size, _p(sc), 0 if e is None else e.size - 1, _p(e)),
                 "oracle_set_tally")

    def run(self, n: int, first: int = 0, seed: int = 1, threads: int = 1, traces: bool = True, sites=None):
        """Returns (tally, traces or None, stats dict, seconds).  sites: n
        source sites (x y z u v w E wgt per row, or a structured array of
        those fields) to start from instead of sampling the source."""
        tally = np.zeros(lib.oracle_tally_size(self.h))
        tr = np.zeros(n, TRACE_DTYPE) if traces else None
        st = OracleStats()
        t0 = time.perf_counter()
        if sites is None:
            self._ck(lib.oracle_run(self.h, first, n, seed, threads, _p(tally), _p(tr), C.byref(st)), "oracle_run")
        else:
            s = np.asarray(sites)
            if s.dtype.names:
                s = np.stack([s[k] for k in ("x", "y", "z", "u", "v", "w", "E", "wgt")], axis=1)
            s = np.ascontiguousarray(s, np.float64).reshape(-1, 8)
            assert s.shape[0] >= n
            self._ck(lib.oracle_run_sites(self.h, first, n, seed, _p(s), threads, _p(tally), _p(tr), C.byref(st)),
                     "oracle_run_sites")
        dt = time.perf_counter() - t0
        return tally, tr, st.as_dict(), dt

    def set_segment_limit(self, n: int) -> None:
        """Segments a history may walk before it ends as stuck (0: default)."""
        self._ck(lib.oracle_set_segment_limit(self.h, n), "oracle_set_segment_limit")

    def segment_limit(self) -> int:
        return lib.oracle_segment_limit(self.h)

    def enable_rays(self, n_rays: int, max_segments: int = 4096) -> None:
        """Record every segment of the first n_rays histories of each run (0: off)."""
        self._ck(lib.oracle_rays_enable(self.h, n_rays, max_segments), "oracle_rays_enable")

    def rays(self) -> np.ndarray:
        """Segments recorded by the last run (RAY_DTYPE), ray by ray."""
        m = C.c_int64()
        self._ck(lib.oracle_rays(self.h, None, 0, C.byref(m)), "oracle_rays")
        out = np.zeros(m.value, RAY_DTYPE)
        self._ck(lib.oracle_rays(self.h, _p(out), out.size, C.byref(m)), "oracle_rays")
        return out

    def eigen(self, n: int, generations: int, inactive: int = 0, seed: int = 1, keff0: float = 0.0,
              watt=(0.0, 0.0), capacity: int = 0, threads: int = 1, initial_source=None, tally: bool = False):
        """k-eigenvalue generations.  Returns (per-generation records
        (GEN_DTYPE), next source (n x 8: x y z u v w E wgt), last sorted
        fission bank (FSITE_DTYPE), active-generation tally SUM or None,
        seconds)."""
        gens = np.zeros(generations, GEN_DTYPE)
        src = np.zeros((n, 8))
        cap = capacity if capacity > 0 else 3 * n
        bank = np.zeros(cap, FSITE_DTYPE)
        m = C.c_int64()
        tsum = np.zeros(lib.oracle_tally_size(self.h)) if tally else None
        init = None if initial_source is None else np.ascontiguousarray(initial_source, np.float64).reshape(n, 8)
        t0 = time.perf_counter()
        self._ck(lib.oracle_eigen_run(self.h, n, generations, inactive, seed, keff0, watt[0], watt[1], cap, threads,
                                      _p(init), _p(gens), _p(src), _p(bank), cap, C.byref(m), _p(tsum)),
                 "oracle_eigen_run")
        dt = time.perf_counter() - t0
        return gens, src, bank[:m.value].copy(), tsum, dt

    def mesh_tables(self):
        nb, pl = C.c_void_p(), C.c_void_p()
        lib.oracle_mesh_info(self.h, C.byref(nb), C.byref(pl))
        nbr = np.ctypeslib.as_array(C.cast(nb, C.POINTER(C.c_int32)), shape=(self.n_tet, 4)).copy()
        planes = np.ctypeslib.as_array(C.cast(pl, C.POINTER(C.c_double)), shape=(self.n_tet, 4, 4)).copy()
        return nbr, planes

    def locate(self, x, u) -> int:
        x = np.ascontiguousarray(x, np.float64)
        u = np.ascontiguousarray(u, np.float64)
        return lib.oracle_locate(self.h, _p(x), _p(u))

    def macro_xs(self, material_index: int, E: float) -> float:
        v = C.c_double()
        self._ck(lib.oracle_macro_xs(self.h, material_index, E, C.byref(v)), "oracle_macro_xs")
        return v.value

    def xs_index(self, nuclide: int, E: float):
        f = C.c_double()
        i = lib.oracle_xs_index(self.h, nuclide, E, C.byref(f))
        return i, f.value


def generator_library() -> C.CDLL:
    """This library's build of the problem generators (mc_gen_* entry
    points), for macaw_gb300.problems.use_generator_library."""
    return lib


def cpu_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def log(x: float) -> float:
    return lib.oracle_log(x)


def quotient(num: float, den: float) -> float:
    """num / den as the walks compute it (Markstein's sequence)."""
    return lib.oracle_quotient(num, den)


def prn(seed: int):
    s = C.c_uint64(seed)
    v = lib.oracle_prn(C.byref(s))
    return v, s.value


def future_seed(n: int, seed: int) -> int:
    return lib.oracle_future_seed(n, seed)


def init_seed(pid: int, master: int, stream: int) -> int:
    return lib.oracle_init_seed(pid, master, stream)
