"""Constants, structures and record layouts of the C ABI (include/macaw_gb300.h).

Importing this module loads no library: problem generators and tools that
only need the layouts (or another build of the generator sources) use it
without the CUDA library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

MC_OK = 0
MC_ERR_ARG, MC_ERR_STATE, MC_ERR_CUDA, MC_ERR_DEVICE, MC_ERR_NOMEM = 1, 2, 3, 4, 5
MC_BC_VACUUM, MC_BC_REFLECT = 0, 1
MC_PREC_FP64, MC_PREC_MIXED = 0, 1
MC_MODE_HISTORY, MC_MODE_EVENT = 0, 1
MC_SRC_POINT, MC_SRC_BOX, MC_SRC_CYLINDERS = 0, 1, 2
MC_SRC_WATT, MC_SRC_MONO = 0, 1
MC_TALLY_BATCH, MC_TALLY_SUM, MC_TALLY_SUM_SQ = 0, 1, 2
MC_EST_TRACKLENGTH, MC_EST_COLLISION = 1, 2
MC_SCORE_FLUX, MC_SCORE_TOTAL, MC_SCORE_SCATTER, MC_SCORE_ABSORPTION = 0, 1, 2, 3
STATUS_NAMES = {1: "leaked", 2: "absorbed", 3: "cutoff", 4: "stuck", 5: "lost", 6: "bad_xs"}


class SourceDesc(C.Structure):
    _fields_ = [("space", C.c_int32), ("energy", C.c_int32),
                ("point", C.c_double * 3), ("box_lo", C.c_double * 3), ("box_hi", C.c_double * 3),
                ("n_cyl", C.c_int32), ("pad", C.c_int32), ("cyl_xy", C.POINTER(C.c_double)),
                ("cyl_r", C.c_double), ("cyl_z0", C.c_double), ("cyl_z1", C.c_double),
                ("watt_a", C.c_double), ("watt_b", C.c_double), ("mono_E", C.c_double)]


class TallyDesc(C.Structure):
    _fields_ = [("estimator", C.c_int32), ("n_scores", C.c_int32), ("scores", C.c_int32 * 4),
                ("n_energy_bins", C.c_int32), ("pad", C.c_int32), ("energy_edges", C.c_void_p)]


class RunDesc(C.Structure):
    _fields_ = [("first_history", C.c_int64), ("n_histories", C.c_int64), ("bank_size", C.c_int64),
                ("seed", C.c_uint64), ("precision", C.c_int32), ("mode", C.c_int32),
                ("block_size", C.c_int32), ("max_seg_per_advance", C.c_int32),
                ("record_traces", C.c_int32), ("accumulate", C.c_int32), ("sort_queue", C.c_int32),
                ("profile", C.c_int32), ("refill", C.c_int32), ("n_batches", C.c_int32), ("graph", C.c_int32),
                ("tail", C.c_int32), ("sites", C.c_void_p), ("batch_sizes", C.c_void_p),
                ("batch_sum_out", C.c_void_p), ("walk_blocks", C.c_int32), ("pad", C.c_int32)]


class EigenDesc(C.Structure):
    _fields_ = [("n_particles", C.c_int64), ("n_batches", C.c_int32), ("n_inactive", C.c_int32),
                ("seed", C.c_uint64), ("precision", C.c_int32), ("mode", C.c_int32), ("bank_size", C.c_int64),
                ("block_size", C.c_int32), ("max_seg_per_advance", C.c_int32), ("sort_queue", C.c_int32),
                ("graph", C.c_int32), ("tail", C.c_int32), ("keff0", C.c_double), ("watt_a", C.c_double), ("watt_b", C.c_double),
                ("fission_bank_capacity", C.c_int64), ("initial_source", C.c_void_p)]


class Job(C.Structure):
    _fields_ = [("ctx", C.c_void_p), ("first_history", C.c_int64), ("n_histories", C.c_int64), ("seed", C.c_uint64)]


class PersistDesc(C.Structure):
    _fields_ = [("precision", C.c_int32), ("block_size", C.c_int32), ("slots", C.c_int32),
                ("record_traces", C.c_int32), ("wait_limit", C.c_int64), ("traces", C.c_void_p)]


class Request(C.Structure):
    _fields_ = [("n_histories", C.c_int64), ("seed", C.c_uint64), ("source", SourceDesc)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("n_hist", "n_seg", "n_coll", "n_leak", "n_absorb", "n_cutoff",
                                        "n_stuck", "n_lost", "n_badxs", "n_fallback", "n_xs", "n_launch")] + \
               [("leak_weight", C.c_double), ("ms_total", C.c_double), ("ms_advance", C.c_double),
                ("n_advance_launch", C.c_int64), ("n_seg_advance", C.c_int64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


TRACE_DTYPE = np.dtype([("id", "<i8"), ("hash", "<u8"), ("status", "<i4"), ("n_seg", "<i4"),
                        ("n_coll", "<i4"), ("elem", "<i4"), ("face", "<i4"), ("pad", "<i4"),
                        ("E", "<f8"), ("x", "<f8"), ("y", "<f8"), ("z", "<f8")])

RAY_SEGMENT_DTYPE = np.dtype([("id", "<i8"), ("segment", "<i4"), ("intersections", "<i4"), ("elem", "<i4"),
                              ("pad", "<i4"), ("start", "<f8", (3,)), ("end", "<f8", (3,)), ("E", "<f8"),
                              ("wgt", "<f8"), ("seed_tracking", "<u8")])

SITE_DTYPE = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("u", "<f8"), ("v", "<f8"),
                       ("w", "<f8"), ("E", "<f8"), ("wgt", "<f8")])

FISSION_SITE_DTYPE = np.dtype([("x", "<f8"), ("y", "<f8"), ("z", "<f8"), ("u", "<f8"), ("v", "<f8"),
                               ("w", "<f8"), ("E", "<f8"), ("wgt", "<f8"), ("parent", "<i8"), ("progeny", "<i4"),
                               ("pad", "<i4")])

EIGEN_GEN_DTYPE = np.dtype([("k_generation", "<f8"), ("k_collision", "<f8"), ("k_absorption", "<f8"),
                            ("keff", "<f8"), ("keff_std", "<f8"), ("leakage", "<f8"), ("n_sites", "<i8"),
                            ("n_seg", "<i8"), ("n_coll", "<i8"), ("ms", "<f8")])

_P = C.c_void_p
_I32, _I64, _U64, _D = C.c_int32, C.c_int64, C.c_uint64, C.c_double

SIGNATURES = {
    "mc_version": ([], C.c_int),
    "mc_ctx_create": ([C.c_int, C.POINTER(_P)], C.c_int),
    "mc_ctx_destroy": ([_P], C.c_int),
    "mc_last_error": ([_P], C.c_char_p),
    "mc_mesh_upload": ([_P, _I64, _P, _I64, _P, _P, _P], C.c_int),
    "mc_bc_set": ([_P, _I32, _I32], C.c_int),
    "mc_nuclide_add": ([_P, _I64, _P, _P, _P, _D, C.POINTER(_I32)], C.c_int),
    "mc_material_add": ([_P, _I32, _I32, _P, _P], C.c_int),
    "mc_nuclide_set_fission": ([_P, _I32, _P], C.c_int),
    "mc_eigen_run": ([_P, C.POINTER(EigenDesc), _P], C.c_int),
    "mc_eigen_source_download": ([_P, _P, _I64], C.c_int),
    "mc_eigen_fission_bank_download": ([_P, _P, _I64, C.POINTER(_I64)], C.c_int),
    "mc_block_material_map": ([_P, _I32, _P, _P], C.c_int),
    "mc_set_hash_bins": ([_P, _I32], C.c_int),
    "mc_source_set": ([_P, C.POINTER(SourceDesc)], C.c_int),
    "mc_run": ([_P, C.POINTER(RunDesc)], C.c_int),
    "mc_sync": ([_P], C.c_int),
    "mc_source_sample": ([_P, _I64, _I64, _U64, _P], C.c_int),
    "mc_ctx_set_stream": ([_P, _P], C.c_int),
    "mc_serve_open": ([_P, _I32, _I64, _I32, _I32], C.c_int),
    "mc_serve_submit": ([_P, C.POINTER(Request), C.POINTER(_I64)], C.c_int),
    "mc_serve_step": ([_P, _I32], C.c_int),
    "mc_serve_poll": ([_P, _P, _I32, C.POINTER(_I32)], C.c_int),
    "mc_serve_result": ([_P, _I64, _P, _I64], C.c_int),
    "mc_serve_status": ([_P, C.POINTER(_I32), C.POINTER(_I32), C.POINTER(_I32)], C.c_int),
    "mc_serve_close": ([_P], C.c_int),
    "mc_run_persistent": ([C.POINTER(PersistDesc), _I32, _P, _P], C.c_int),
    "mc_run_noalloc": ([_P, C.POINTER(RunDesc), _P, _P], C.c_int),
    "mc_app_run": ([C.c_char_p, C.c_int, C.c_char_p, C.c_char_p, _I64], C.c_int),
    "mc_app_check": ([C.c_char_p, C.c_char_p, _I64], C.c_int),
    "mc_tally_download": ([_P, _I32, _P, _I64], C.c_int),
    "mc_tally_configure": ([_P, C.c_void_p], C.c_int),
    "mc_set_2d": ([_P, _I32, _D], C.c_int),
    "mc_set_segment_limit": ([_P, _I64], C.c_int),
    "mc_segment_limit": ([_P, C.POINTER(_I64)], C.c_int),
    "mc_exodus_read_sizes": ([C.c_char_p, C.POINTER(_I64), C.POINTER(_I64), C.c_char_p, _I64], C.c_int),
    "mc_exodus_read": ([C.c_char_p, _P, _P, _P, _P, C.c_char_p, _I64], C.c_int),
    "mc_rays_enable": ([_P, _I32, _I32], C.c_int),
    "mc_rays_download": ([_P, _P, _I64, C.POINTER(_I64)], C.c_int),
    "mc_exodus_write_rays": ([C.c_char_p, _P, _I64, _I64], C.c_int),
    "mc_exodus_write": ([C.c_char_p, C.c_char_p, _I64, _P, _I64, _P, _P, _P, _I32, _P, _P, _D], C.c_int),
    "mc_tally_size": ([_P, C.POINTER(_I64)], C.c_int),
    "mc_tally_reset": ([_P], C.c_int),
    "mc_tally_clear": ([_P, _I32], C.c_int),
    "mc_autotune": ([_P, C.POINTER(RunDesc), _I64, C.POINTER(RunDesc), C.POINTER(_D)], C.c_int),
    "mc_trace_download": ([_P, _P, _I64], C.c_int),
    "mc_stats_get": ([_P, C.POINTER(Stats)], C.c_int),
    "mc_batches_done": ([_P, C.POINTER(_I64)], C.c_int),
    "mc_gen_box_sizes": ([_I32, _I32, _I32, C.POINTER(_I64), C.POINTER(_I64)], C.c_int),
    "mc_gen_box": ([_I32, _I32, _I32, _P, _P, _P, _P, _P, _P], C.c_int),
    "mc_gen_cube_sizes": ([_I32, C.POINTER(_I64), C.POINTER(_I64)], C.c_int),
    "mc_gen_cube": ([_I32, _D, _P, _P, _P, _P], C.c_int),
    "mc_gen_lattice_sizes": ([_I32, _I32, _I32, _I32, _I32, C.POINTER(_I64), C.POINTER(_I64)], C.c_int),
    "mc_gen_lattice": ([_I32, _I32, _I32, _I32, _I32, _D, _D, _D, _D, _P, _P, _P, _P], C.c_int),
    "mc_gen_core_sizes": ([_I32, _I32, _I32, _I32, _D, _D, C.POINTER(_I64), C.POINTER(_I64), C.POINTER(_I64)], C.c_int),
    "mc_gen_core": ([_I32, _I32, _I32, _I32, _D, _D, _D, _D, _D, _P, _P, _P, _P, _P], C.c_int),
    "mc_gen_nuclide": ([_U64, _I32, _I64, _D, _D, _I32, _P, _P, _P, C.POINTER(_D)], C.c_int),
    "mc_gen_densities": ([_U64, _I32, _I32, _D, _D, _P], C.c_int),
}
