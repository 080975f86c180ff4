"""The C-ABI library: exports, host-only entry points, argument checks (no GPU)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from macaw_gb300 import _lib, problems

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(mc_\w+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    names = declared_symbols()
    assert "mc_run" in names and "mc_mesh_upload" in names and len(names) >= 20
    for n in names:
        assert hasattr(_lib.lib, n), f"{n} declared in include/ but not exported"
    # and every binding the package uses is declared
    for n in _lib.SIGNATURES:
        assert n in names, f"{n} bound in _lib.py but not declared in include/"


def _header_sizes(tmp_path):
    """sizeof and offsetof of the ABI structs as a C compiler lays them out
    from include/macaw_gb300.h."""
    import shutil
    import subprocess
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    inc = ROOT / "include"
    src = tmp_path / "sizes.c"
    structs = ["mc_source_desc", "mc_site", "mc_fission_site", "mc_run_desc", "mc_trace", "mc_stats",
               "mc_tally_desc", "mc_ray_segment", "mc_eigen_desc", "mc_eigen_gen", "mc_job", "mc_persist_desc"]
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "macaw_gb300.h"\nint main(void){\n' +
                   "".join(f'printf("{n} %zu\\n", sizeof({n}));\n' for n in structs) +
                   'printf("batch_sum_out %zu\\n", offsetof(mc_run_desc, batch_sum_out));\nreturn 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run([cc, "-I", str(inc), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return {k: int(v) for k, v in (line.split() for line in out.splitlines())}


def test_struct_layouts_match_header_sizes(tmp_path):
    h = _header_sizes(tmp_path)
    assert C.sizeof(_lib.SourceDesc) == h["mc_source_desc"]
    assert C.sizeof(_lib.RunDesc) == h["mc_run_desc"]
    assert _lib.RunDesc.batch_sum_out.offset == h["batch_sum_out"]
    assert C.sizeof(_lib.EigenDesc) == h["mc_eigen_desc"]
    assert C.sizeof(_lib.Job) == h["mc_job"]
    assert C.sizeof(_lib.PersistDesc) == h["mc_persist_desc"]
    assert C.sizeof(_lib.TallyDesc) == h["mc_tally_desc"]
    assert C.sizeof(_lib.Stats) == h["mc_stats"]
    assert _lib.TRACE_DTYPE.itemsize == h["mc_trace"]
    assert _lib.SITE_DTYPE.itemsize == h["mc_site"]
    assert _lib.FISSION_SITE_DTYPE.itemsize == h["mc_fission_site"]
    assert _lib.RAY_SEGMENT_DTYPE.itemsize == h["mc_ray_segment"]
    assert _lib.EIGEN_GEN_DTYPE.itemsize == h["mc_eigen_gen"]


def test_version():
    assert _lib.lib.mc_version() >= 1


def test_cube_generator_counts_and_sidesets():
    xyz, tv, blk, bid = problems.cube_mesh(4, 4.0)
    assert xyz.shape == (125, 3) and tv.shape == (384, 4)
    # each outer face of the cube carries 4*4*2 triangles, one sideset per face
    ids, counts = np.unique(bid[bid >= 0], return_counts=True)
    assert list(ids) == [0, 1, 2, 3, 4, 5]
    assert np.all(counts == 32)
    # every tet has positive volume
    P = xyz[tv]
    vol = np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0])
    assert np.all(np.abs(vol) > 1e-12)
    assert np.isclose(np.abs(vol).sum() / 6.0, 64.0)


def test_lattice_generator_volume_and_blocks():
    xyz, tv, blk, bid = problems.lattice_mesh(nx=2, ny=3, nz=2, height=5.0)
    P = xyz[tv]
    vol = np.abs(np.einsum("ij,ij->i", np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0]), P[:, 3] - P[:, 0])) / 6
    assert np.isclose(vol.sum(), 2 * 1.26 * 3 * 1.26 * 5.0, rtol=1e-12)
    assert set(np.unique(blk)) == {1, 2, 3}
    ids = np.unique(bid[bid >= 0])
    assert list(ids) == [0, 1, 2, 3, 4, 5]
    # fuel area fraction close to the 16-gon inscribed in r=0.41
    fuel = vol[blk == 1].sum() / 5.0 / 6
    poly = 0.5 * 16 * 0.41**2 * np.sin(2 * np.pi / 16)
    assert np.isclose(fuel, poly, rtol=1e-9)


def test_full_size_lattice_is_about_two_million_tets():
    nv, nt = C.c_int64(), C.c_int64()
    assert _lib.lib.mc_gen_lattice_sizes(17, 17, 21, 16, 2, C.byref(nv), C.byref(nt)) == 0
    assert nt.value == 2039184


def test_generators_are_deterministic():
    a = problems.make_nuclide(5, 3, 1000)
    b = problems.make_nuclide(5, 3, 1000)
    assert np.array_equal(a.E, b.E) and np.array_equal(a.sig_t, b.sig_t) and a.awr == b.awr
    c = problems.make_nuclide(5, 4, 1000)
    assert not np.array_equal(a.sig_t, c.sig_t)
    assert np.all(np.diff(a.E) > 0) and a.E[0] == 1e-5 and a.E[-1] == 2e7
    assert np.all(a.sig_s <= a.sig_t) and np.all(a.sig_t > 0)


def test_generator_rejects_bad_arguments():
    out = np.zeros(4)
    assert _lib.lib.mc_gen_nuclide(1, 0, 1, 1e-5, 2e7, 0, _lib.ptr(out), _lib.ptr(out), _lib.ptr(out),
                                   C.byref(C.c_double())) != 0
    nv, nt = C.c_int64(), C.c_int64()
    assert _lib.lib.mc_gen_lattice_sizes(2, 2, 2, 12, 2, C.byref(nv), C.byref(nt)) != 0  # n_sec % 8


def test_context_creation_fails_loudly_without_gpu():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    assert _lib.lib.mc_ctx_create(0, C.byref(h)) != 0
    from macaw_gb300 import MCError, Tracker
    with pytest.raises(MCError):
        Tracker(0)
