"""Exodus II files (mc_exodus_write, mc_exodus_read).

    from macaw_gb300 import exodus
    exodus.write("flux.e", problem, {"flux": values})
    xyz, tet_vtx, tet_block, tet_side_bid = exodus.read_mesh("mesh.e")

write stores the problem's tet mesh (one TETRA4 block per subdomain, side
sets from its boundary ids) with one element variable per field, as MOOSE
writes a MaCaw run's AuxVariables; read_mesh reads a tet mesh as MOOSE's
FileMeshGenerator does (elements in block order).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import MCError, lib, ptr


def write(path: str, problem, fields: dict, time: float = 1.0, title: str = "macaw_gb300") -> None:
    xyz = np.ascontiguousarray(problem.xyz, np.float64)
    tv = np.ascontiguousarray(problem.tet_vtx, np.int32)
    blk = np.ascontiguousarray(problem.tet_block, np.int32)
    names = list(fields)
    vals = np.ascontiguousarray(np.stack([np.asarray(fields[k], np.float64) for k in names])
                                if names else np.zeros((0, tv.shape[0])))
    if vals.shape != (len(names), tv.shape[0]):
        raise ValueError("each field needs one value per element")
    cnames = (C.c_char_p * max(1, len(names)))(*[n.encode() for n in names])
    bid = None if problem.tet_side_bid is None else np.ascontiguousarray(problem.tet_side_bid, np.int32)
    rc = lib.mc_exodus_write(path.encode(), title.encode(), xyz.shape[0], ptr(xyz), tv.shape[0], ptr(tv),
                             ptr(blk), ptr(bid), len(names), C.cast(cnames, C.c_void_p), ptr(vals), float(time))
    if rc != 0:
        raise MCError(rc, f"mc_exodus_write({path}) failed")


def read_mesh(path: str):
    """(xyz, tet_vtx, tet_block, tet_side_bid) of an Exodus II tet mesh."""
    nv, nt = C.c_int64(), C.c_int64()
    err = C.create_string_buffer(512)
    rc = lib.mc_exodus_read_sizes(path.encode(), C.byref(nv), C.byref(nt), err, 512)
    if rc != 0:
        raise MCError(rc, err.value.decode())
    xyz = np.zeros((nv.value, 3))
    tv = np.zeros((nt.value, 4), np.int32)
    blk = np.zeros(nt.value, np.int32)
    bid = np.zeros((nt.value, 4), np.int32)
    rc = lib.mc_exodus_read(path.encode(), ptr(xyz), ptr(tv), ptr(blk), ptr(bid), err, 512)
    if rc != 0:
        raise MCError(rc, err.value.decode())
    return xyz, tv, blk, bid


def write_rays(path: str, segments: np.ndarray, first_history: int = 0) -> None:
    """Recorded ray segments (Tracker.rays()) as a RayTracingExodus file."""
    from ._lib import RAY_SEGMENT_DTYPE
    seg = np.ascontiguousarray(segments, RAY_SEGMENT_DTYPE)
    rc = lib.mc_exodus_write_rays(path.encode(), ptr(seg), seg.size, first_history)
    if rc != 0:
        raise MCError(rc, f"mc_exodus_write_rays({path}) failed")
