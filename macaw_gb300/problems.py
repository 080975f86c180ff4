"""Synthetic fixed-source problems (meshes, cross sections, sources).

The reference's inputs (BEAVRS meshes, ENDF/HDF5 nuclear data) are not
shipped with it and cannot be downloaded here, so problems are generated
from one seed by the library's own generators (mc_gen_*), which produce
bit-identical tables on every host architecture.

cube_problem     -- 20 cm cube, 20^3 hexes x 6 tets (48,000 tets), one
                    material of 10 nuclides, 10,000-point grids, point source
                    at the centre, Watt spectrum, vacuum boundary.
lattice_problem  -- 17x17 pin cells, pitch 1.26 cm, 50 cm tall, fuel/clad/
                    moderator rings (15/4/3 nuclides, 20,000-point grids),
                    about 2.0M tets, uniform source in the fuel cylinders.
eigen_lattice_problem -- the pin lattice as a k-eigenvalue problem:
                    fissionable fuel nuclides (nu*sigma_f a fixed share of
                    their absorption), reflective sides, vacuum top and
                    bottom.
study_box_problem -- the mesh of the reference's study test (a 5x5x1 box of
                    hexes over [-5, 5]^3 cut into tets, centre hex in block 1,
                    reflective on every side) with transparent materials,
                    for pure-geometry walks.
core_problem     -- cylindrical core, radius 180 cm, 400 cm tall: 193
                    assemblies of 17x17 pin cells plus a reflector of whole
                    cells, 6 axial layers (about 41M tets); 200 materials of
                    5-40 nuclides drawn from a pool of 300 (30,000-point
                    grids, up to 60 peaks); uniform source in every fuel
                    cylinder.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from ._abi import MC_BC_REFLECT, MC_BC_VACUUM, MC_SRC_CYLINDERS, MC_SRC_POINT, MC_SRC_WATT, SIGNATURES

_GEN = None  # library whose mc_gen_* entry points build the problems


def use_generator_library(handle) -> None:
    """Builds problems with another compiled copy of the generator sources
    (macaw_gb300/csrc/mc_gen.cpp) exposing the same mc_gen_* entry points,
    instead of the tracker's library (None: back to the tracker's)."""
    global _GEN
    if handle is not None:
        for name, (args, res) in SIGNATURES.items():
            if name.startswith("mc_gen_"):
                fn = getattr(handle, name)
                fn.argtypes = args
                fn.restype = res
    _GEN = handle


def _lib():
    if _GEN is not None:
        return _GEN
    from ._lib import lib
    return lib


def ptr(a):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays passed to the C ABI must be contiguous"
    return C.c_void_p(a.ctypes.data)

WATT_A = 0.988e6   # eV
WATT_B = 2.249e-6  # 1/eV
E_MIN, E_MAX = 1.0e-5, 2.0e7  # eV


@dataclass
class Nuclide:
    E: np.ndarray
    sig_t: np.ndarray
    sig_s: np.ndarray
    awr: float
    nu_sig_f: np.ndarray | None = None  # nu*sigma_f per point; None: not fissionable


@dataclass
class Material:
    id: int
    nuclides: np.ndarray  # int32 indices into Problem.nuclides
    densities: np.ndarray  # atom/b-cm


@dataclass
class Source:
    space: int = MC_SRC_POINT
    energy: int = MC_SRC_WATT
    point: tuple = (0.0, 0.0, 0.0)
    box_lo: tuple = (0.0, 0.0, 0.0)
    box_hi: tuple = (0.0, 0.0, 0.0)
    cyl_xy: np.ndarray | None = None
    cyl_r: float = 0.0
    cyl_z0: float = 0.0
    cyl_z1: float = 0.0
    watt_a: float = WATT_A
    watt_b: float = WATT_B
    mono_E: float = 0.0


@dataclass
class TallyDef:
    """OpenMCTally's estimator, scores and energy filter for the element
    tally (MC_EST_*, MC_SCORE_*; energy_edges None: no energy filter)."""
    estimator: int = 1
    scores: tuple = (0,)
    energy_edges: np.ndarray | None = None


@dataclass
class Problem:
    name: str
    xyz: np.ndarray
    tet_vtx: np.ndarray
    tet_block: np.ndarray
    tet_side_bid: np.ndarray
    nuclides: list
    materials: list
    blocks: np.ndarray
    block_materials: np.ndarray
    source: Source
    bcs: dict = field(default_factory=dict)  # boundary id -> MC_BC_*
    hash_bins: int = 8000
    tally: TallyDef | None = None  # None: track-length flux per element
    z_2d: float | None = None      # 2-D mode (CollisionKernel z_coord): None for 3-D

    @property
    def n_tet(self) -> int:
        return int(self.tet_vtx.shape[0])

    def footprint_bytes(self) -> int:
        pts = sum(n.E.size for n in self.nuclides)
        return self.n_tet * (128 + 64 + 16 + 4 + 3 * 8) + pts * 32


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise RuntimeError(f"{what} failed with code {rc}")


def cube_mesh(n: int = 20, L: float = 20.0):
    nv, nt = C.c_int64(), C.c_int64()
    _check(_lib().mc_gen_cube_sizes(n, C.byref(nv), C.byref(nt)), "mc_gen_cube_sizes")
    xyz = np.zeros((nv.value, 3), np.float64)
    tv = np.zeros((nt.value, 4), np.int32)
    blk = np.zeros(nt.value, np.int32)
    bid = np.zeros((nt.value, 4), np.int32)
    _check(_lib().mc_gen_cube(n, L, ptr(xyz), ptr(tv), ptr(blk), ptr(bid)), "mc_gen_cube")
    return xyz, tv, blk, bid


def box_mesh(nx: int, ny: int, nz: int, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0)):
    nv, nt = C.c_int64(), C.c_int64()
    _check(_lib().mc_gen_box_sizes(nx, ny, nz, C.byref(nv), C.byref(nt)), "mc_gen_box_sizes")
    xyz = np.zeros((nv.value, 3), np.float64)
    tv = np.zeros((nt.value, 4), np.int32)
    blk = np.zeros(nt.value, np.int32)
    bid = np.zeros((nt.value, 4), np.int32)
    lo_a = np.ascontiguousarray(lo, np.float64)
    hi_a = np.ascontiguousarray(hi, np.float64)
    _check(_lib().mc_gen_box(nx, ny, nz, ptr(lo_a), ptr(hi_a), ptr(xyz), ptr(tv), ptr(blk), ptr(bid)), "mc_gen_box")
    return xyz, tv, blk, bid


def lattice_mesh(nx: int = 17, ny: int = 17, nz: int = 21, n_sec: int = 16, n_fuel_rings: int = 2,
                 pitch: float = 1.26, height: float = 50.0, r_fuel: float = 0.41, r_clad: float = 0.475):
    nv, nt = C.c_int64(), C.c_int64()
    _check(_lib().mc_gen_lattice_sizes(nx, ny, nz, n_sec, n_fuel_rings, C.byref(nv), C.byref(nt)),
           "mc_gen_lattice_sizes")
    xyz = np.zeros((nv.value, 3), np.float64)
    tv = np.zeros((nt.value, 4), np.int32)
    blk = np.zeros(nt.value, np.int32)
    bid = np.zeros((nt.value, 4), np.int32)
    _check(_lib().mc_gen_lattice(nx, ny, nz, n_sec, n_fuel_rings, pitch, height, r_fuel, r_clad,
                              ptr(xyz), ptr(tv), ptr(blk), ptr(bid)), "mc_gen_lattice")
    return xyz, tv, blk, bid


def core_mesh(pins: int = 17, nz: int = 6, n_sec: int = 8, n_fuel_rings: int = 1, pitch: float = 1.26,
              height: float = 400.0, r_fuel: float = 0.41, r_clad: float = 0.475, radius: float = 180.0):
    nv, nt, npn = C.c_int64(), C.c_int64(), C.c_int64()
    _check(_lib().mc_gen_core_sizes(pins, nz, n_sec, n_fuel_rings, pitch, radius, C.byref(nv), C.byref(nt),
                                 C.byref(npn)), "mc_gen_core_sizes")
    xyz = np.zeros((nv.value, 3), np.float64)
    tv = np.zeros((nt.value, 4), np.int32)
    blk = np.zeros(nt.value, np.int32)
    bid = np.zeros((nt.value, 4), np.int32)
    pins_xy = np.zeros((npn.value, 2), np.float64)
    _check(_lib().mc_gen_core(pins, nz, n_sec, n_fuel_rings, pitch, height, r_fuel, r_clad, radius, ptr(xyz), ptr(tv),
                           ptr(blk), ptr(bid), ptr(pins_xy)), "mc_gen_core")
    return xyz, tv, blk, bid, pins_xy


def _splitmix(x: int) -> int:
    """splitmix64 finaliser (integer-only, identical on every host)."""
    x = (x + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    x = ((x ^ (x >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return x ^ (x >> 31)


def make_nuclide(seed: int, index: int, n_pts: int, n_peaks: int = 20,
                 E_min: float = E_MIN, E_max: float = E_MAX) -> Nuclide:
    E = np.zeros(n_pts)
    st = np.zeros(n_pts)
    ss = np.zeros(n_pts)
    awr = C.c_double()
    _check(_lib().mc_gen_nuclide(seed, index, n_pts, E_min, E_max, n_peaks, ptr(E), ptr(st), ptr(ss),
                              C.byref(awr)), "mc_gen_nuclide")
    return Nuclide(E, st, ss, awr.value)


def make_densities(seed: int, index: int, n: int, lo: float = 1e-4, hi: float = 5e-2) -> np.ndarray:
    out = np.zeros(n)
    _check(_lib().mc_gen_densities(seed, index, n, lo, hi, ptr(out)), "mc_gen_densities")
    return out


def cube_problem(n: int = 20, L: float = 20.0, n_nuc: int = 10, n_pts: int = 10000, n_peaks: int = 20,
                 seed: int = 20240611) -> Problem:
    """The 48,000-tet cube of the plain FP64 configuration (at n=20)."""
    xyz, tv, blk, bid = cube_mesh(n, L)
    nucs = [make_nuclide(seed, i, n_pts, n_peaks) for i in range(n_nuc)]
    mat = Material(1, np.arange(n_nuc, dtype=np.int32), make_densities(seed, 0, n_nuc))
    src = Source(space=MC_SRC_POINT, point=(L / 2, L / 2, L / 2))
    return Problem(f"cube{n}", xyz, tv, blk, bid, nucs, [mat], np.array([0], np.int32),
                   np.array([1], np.int32), src, {b: MC_BC_VACUUM for b in range(6)})


def study_box_problem(sigma_b: float = 1e-20, density: float = 1e-4) -> Problem:
    """The mesh of MaCaw's study test (test/tests/study/openmc_study.i:1-22):
    GeneratedMeshGenerator 5 x 5 x 1 hexes over [-5, 5]^3, each hex cut
    into six Kuhn tets; SubdomainBoundingBoxGenerator puts the hex inside
    [-1, 1]^3 into block 1, the rest stays in block 0; ReflectRayBC on all
    six sides (:49-54); blocks 0 and 1 map to materials 1 and 2 (CollisionKernel
    `blocks = "0 1 2"`, `materials = "1 2 3"`, :42-47).  The materials are
    transparent (one nuclide of sigma_b barn at `density`), so histories
    fly without colliding: the walk and the reflections alone set their
    paths."""
    xyz, tv, blk, bid = box_mesh(5, 5, 1, (-5.0, -5.0, -5.0), (5.0, 5.0, 5.0))
    # hex centres (the six Kuhn tets of a hex are consecutive; their
    # centroids average to the hex centre), as SubdomainBoundingBoxGenerator
    # tests element centres against the box
    hc = np.repeat(xyz[tv].mean(axis=1).reshape(-1, 6, 3).mean(axis=1), 6, axis=0)
    blk[:] = np.where(np.all(np.abs(hc) < 1.0, axis=1), 1, 0).astype(np.int32)
    E = np.array([E_MIN, E_MAX])
    nuc = Nuclide(E, np.full(2, sigma_b), np.full(2, sigma_b), 1.0)
    mats = [Material(m, np.array([0], np.int32), np.array([density])) for m in (1, 2, 3)]
    src = Source(space=MC_SRC_POINT, point=(0.0, 0.0, 0.0))
    return Problem("study_box", xyz, tv, blk, bid, [nuc], mats, np.array([0, 1, 2], np.int32),
                   np.array([1, 2, 3], np.int32), src, {b: MC_BC_REFLECT for b in range(6)}, hash_bins=16)


def lattice_problem(nx: int = 17, ny: int = 17, nz: int = 21, n_sec: int = 16, n_fuel_rings: int = 2,
                    pitch: float = 1.26, height: float = 50.0, n_pts: int = 20000, n_peaks: int = 20,
                    nuclides_per_material=(15, 4, 3), seed: int = 20240611) -> Problem:
    """17x17 pin lattice (about 2.0M tets at the defaults): blocks 1 fuel,
    2 clad, 3 moderator mapped to materials 1, 2, 3."""
    xyz, tv, blk, bid = lattice_mesh(nx, ny, nz, n_sec, n_fuel_rings, pitch, height)
    nucs, mats = [], []
    k = 0
    for m, cnt in enumerate(nuclides_per_material):
        idx = []
        for _ in range(cnt):
            nucs.append(make_nuclide(seed, k, n_pts, n_peaks))
            idx.append(k)
            k += 1
        mats.append(Material(m + 1, np.array(idx, np.int32), make_densities(seed, m, cnt)))
    cx = (np.arange(nx) + 0.5) * pitch
    cy = (np.arange(ny) + 0.5) * pitch
    centres = np.array([(x, y) for y in cy for x in cx], np.float64)
    src = Source(space=MC_SRC_CYLINDERS, cyl_xy=np.ascontiguousarray(centres), cyl_r=0.41,
                 cyl_z0=0.0, cyl_z1=height)
    return Problem(f"lattice{nx}x{ny}x{nz}", xyz, tv, blk, bid, nucs, mats,
                   np.array([1, 2, 3], np.int32), np.array([1, 2, 3], np.int32), src,
                   {b: MC_BC_VACUUM for b in range(6)})


def core_problem(pins: int = 17, nz: int = 6, n_sec: int = 8, n_fuel_rings: int = 1, pitch: float = 1.26,
                 height: float = 400.0, radius: float = 180.0, n_pool: int = 300, n_pts: int = 30000,
                 max_peaks: int = 60, nuclides_per_material=(5, 40), seed: int = 20240611) -> Problem:
    """Cylindrical core (about 41M tets at the defaults).  Blocks 1..193 are
    the fuel of each assembly, 194 clad, 195 moderator, 196..200 reflector
    sectors; block b maps to material b.  Material b holds a count drawn
    uniformly from `nuclides_per_material` of distinct nuclides out of a
    pool of `n_pool`; nuclide k has 1 + (k mod max_peaks) resonance peaks.
    Vacuum on every sideset (bottom 0, top 5, radial 6)."""
    xyz, tv, blk, bid, pins_xy = core_mesh(pins, nz, n_sec, n_fuel_rings, pitch, height, radius=radius)
    nucs = [make_nuclide(seed, k, n_pts, 1 + k % max_peaks) for k in range(n_pool)]
    lo, hi = nuclides_per_material
    mats = []
    for b in range(1, 201):
        h = _splitmix(seed * 1000003 + b)
        cnt = min(lo + h % (hi - lo + 1), n_pool)
        chosen, j = [], 0
        while len(chosen) < cnt:
            k = _splitmix(h + 7919 * j) % n_pool
            j += 1
            if k not in chosen:
                chosen.append(k)
        mats.append(Material(b, np.array(sorted(chosen), np.int32), make_densities(seed, 1000 + b, cnt)))
    blocks = np.arange(1, 201, dtype=np.int32)
    src = Source(space=MC_SRC_CYLINDERS, cyl_xy=np.ascontiguousarray(pins_xy), cyl_r=0.41 * pitch / 1.26,
                 cyl_z0=0.0, cyl_z1=height)
    return Problem(f"core{pins}x{nz}", xyz, tv, blk, bid, nucs, mats, blocks, blocks.copy(), src,
                   {b: MC_BC_VACUUM for b in range(7)})


def lattice_2d_problem(nx: int = 17, ny: int = 17, n_sec: int = 16, n_fuel_rings: int = 2, pitch: float = 1.26,
                       thickness: float = 1.0, n_pts: int = 20000, n_peaks: int = 20,
                       nuclides_per_material=(15, 4, 3), seed: int = 20240611) -> Problem:
    """2-D pin lattice (CollisionKernel z_coord): the lattice's 2-D mesh
    extruded into one layer of tets of the given thickness, histories in
    the mid-plane, reflective top and bottom (never reached: directions
    stay in the plane)."""
    p = lattice_problem(nx, ny, 1, n_sec, n_fuel_rings, pitch, thickness, n_pts, n_peaks, nuclides_per_material,
                        seed)
    p.name = f"lattice2d{nx}x{ny}"
    p.z_2d = thickness / 2
    p.bcs[0] = p.bcs[5] = MC_BC_REFLECT
    return p


def add_fission(nuc: Nuclide, nu: float = 2.43, fission_share: float = 0.8) -> Nuclide:
    """Makes a nuclide fissionable: nu*sigma_f(E) = nu * fission_share *
    sigma_a(E), sigma_a = sigma_t - sigma_s at every grid point."""
    nuc.nu_sig_f = (nu * fission_share) * (nuc.sig_t - nuc.sig_s)
    return nuc


def eigen_lattice_problem(nx: int = 17, ny: int = 17, nz: int = 21, n_sec: int = 16, n_fuel_rings: int = 2,
                          pitch: float = 1.26, height: float = 50.0, n_pts: int = 20000, n_peaks: int = 20,
                          nuclides_per_material=(15, 4, 3), scatter_b: float = 2.0, absorb_b: float = 0.5,
                          nu: float = 2.43, fission_share: float = 0.6, seed: int = 20240611) -> Problem:
    """k-eigenvalue pin lattice (about 2.0M tets at the defaults, k near 1):
    the lattice's tables plus a constant scattering (scatter_b) and
    absorption (absorb_b) cross section on every nuclide, so that fission
    neutrons collide within a few pin cells; every fuel nuclide is
    fissionable (add_fission); reflective sides (sidesets 1-4), vacuum top
    and bottom (0, 5).  The first generation starts from the uniform source
    in the fuel cylinders."""
    p = lattice_problem(nx, ny, nz, n_sec, n_fuel_rings, pitch, height, n_pts, n_peaks, nuclides_per_material, seed)
    p.name = f"eigen_lattice{nx}x{ny}x{nz}"
    for n in p.nuclides:
        n.sig_s = n.sig_s + scatter_b
        n.sig_t = n.sig_t + (scatter_b + absorb_b)
    for k in p.materials[0].nuclides:
        add_fission(p.nuclides[int(k)], nu, fission_share)
    for b in (1, 2, 3, 4):
        p.bcs[b] = MC_BC_REFLECT
    return p
