"""Exodus II output, read back with scipy's netCDF reader.

The file must carry what an Exodus reader looks for: the coordinates, one
TETRA4 block per subdomain with 1-based connectivity and the block ids,
the element variable names, one time step and each variable's values per
block in mesh order.
"""
import numpy as np
import pytest

from macaw_gb300 import exodus, problems

netcdf = pytest.importorskip("scipy.io").netcdf_file


def _chars(a):
    return [bytes(r).rstrip(b"\0").decode() for r in np.asarray(a)]


def test_lattice_fields_round_trip(tmp_path):
    p = problems.lattice_problem(nx=2, ny=2, nz=2, height=4.0, n_pts=50)
    rng = np.random.default_rng(1)
    flux = rng.random(p.n_tet)
    power = np.arange(p.n_tet, dtype=np.float64)
    path = str(tmp_path / "lat.e")
    exodus.write(path, p, {"flux": flux, "power": power}, time=2.5)
    with netcdf(path, "r", mmap=False) as f:
        assert f.dimensions["num_nodes"] == p.xyz.shape[0]
        assert f.dimensions["num_elem"] == p.n_tet
        blocks = np.unique(p.tet_block)
        assert f.dimensions["num_el_blk"] == blocks.size
        assert np.array_equal(f.variables["eb_prop1"][:], blocks)
        for k, c in enumerate("xyz"):
            assert np.array_equal(f.variables["coord" + c][:], p.xyz[:, k])
        assert _chars(f.variables["name_elem_var"][:]) == ["flux", "power"]
        assert f.variables["time_whole"][:].tolist() == [2.5]
        for i, b in enumerate(blocks):
            conn = f.variables[f"connect{i + 1}"]
            assert conn.elem_type == b"TETRA4"
            members = np.nonzero(p.tet_block == b)[0]
            assert np.array_equal(conn[:] - 1, p.tet_vtx[members])
            assert np.array_equal(f.variables[f"vals_elem_var1eb{i + 1}"][0], flux[members])
            assert np.array_equal(f.variables[f"vals_elem_var2eb{i + 1}"][0], power[members])


def test_mesh_round_trip_with_side_sets(tmp_path):
    p = problems.lattice_problem(nx=2, ny=2, nz=2, height=4.0, n_pts=50)
    path = str(tmp_path / "mesh.e")
    exodus.write(path, p, {})
    xyz, tv, blk, bid = exodus.read_mesh(path)
    order = np.argsort(p.tet_block, kind="stable")  # the file numbers elements block by block
    assert np.array_equal(xyz, p.xyz)
    assert np.array_equal(tv, p.tet_vtx[order]) and np.array_equal(blk, p.tet_block[order])
    # boundary faces keep their side set ids; interior faces have none
    from oracle import oracle as O
    nbr, _ = O.Oracle(p).mesh_tables()
    ref = np.where(nbr < 0, p.tet_side_bid, -1)[order]
    assert np.array_equal(bid, ref)
    assert set(np.unique(bid[bid >= 0])) == {0, 1, 2, 3, 4, 5}


def test_core_round_trip_keeps_the_radial_side_set(tmp_path):
    xyz, tv, blk, bid, _ = problems.core_mesh(pins=2, nz=2, height=6.0, radius=22.0)
    p = problems.Problem("c", xyz, tv, blk, bid, [], [], np.zeros(0, np.int32), np.zeros(0, np.int32),
                         problems.Source())
    path = str(tmp_path / "core.e")
    exodus.write(path, p, {"blk": blk.astype(np.float64)})
    x2, t2, b2, s2 = exodus.read_mesh(path)
    order = np.argsort(blk, kind="stable")
    assert np.array_equal(t2, tv[order]) and np.array_equal(b2, blk[order])
    assert set(np.unique(s2[s2 >= 0])) == {0, 5, 6}


def test_non_tet_files_are_refused(tmp_path):
    from macaw_gb300._lib import MCError
    path = tmp_path / "x.e"
    path.write_bytes(b"not netcdf")
    with pytest.raises(MCError, match="netCDF"):
        exodus.read_mesh(str(path))


def _scipy_exodus(path, conn, elem_type, xyz, coord_2d=False):
    """A minimal Exodus file written by scipy's own netCDF writer (classic format)."""
    with netcdf(path, "w", version=1) as f:
        f.createDimension("num_dim", 3)
        f.createDimension("num_nodes", xyz.shape[0])
        f.createDimension("num_elem", conn.shape[0])
        f.createDimension("num_el_blk", 1)
        f.createDimension("num_el_in_blk1", conn.shape[0])
        f.createDimension("num_nod_per_el1", conn.shape[1])
        if coord_2d:
            c = f.createVariable("coord", "d", ("num_dim", "num_nodes"))
            c[:] = xyz.T
        else:
            for k, n in enumerate("xyz"):
                f.createVariable("coord" + n, "d", ("num_nodes",))[:] = xyz[:, k]
        v = f.createVariable("connect1", "i", ("num_el_in_blk1", "num_nod_per_el1"))
        v[:] = conn + 1
        v.elem_type = elem_type
        f.createVariable("eb_prop1", "i", ("num_el_blk",))[:] = [7]


def test_reads_files_from_another_netcdf_writer(tmp_path):
    xyz = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0, 0, 1], [1, 1, 1]], np.float64)
    conn = np.array([[0, 1, 2, 3], [1, 2, 3, 4]], np.int32)
    path = str(tmp_path / "s.e")
    _scipy_exodus(path, conn, "TETRA4", xyz, coord_2d=True)
    x2, t2, b2, s2 = exodus.read_mesh(path)
    assert np.array_equal(x2, xyz) and np.array_equal(t2, conn) and np.all(b2 == 7) and np.all(s2 == -1)
    hexes = np.arange(8, dtype=np.int32)[None, :]
    _scipy_exodus(path, hexes, "HEX8", np.random.default_rng(0).random((8, 3)))
    from macaw_gb300._lib import MCError
    with pytest.raises(MCError, match="only 4-node tetrahedra"):
        exodus.read_mesh(path)


REF_RAY_VARS = ["aux_energy", "aux_id", "aux_n_progeny", "aux_particle_type", "aux_seed_URR", "aux_seed_source",
                "aux_seed_tracking", "aux_weight", "intersections", "ray_id"]


def test_ray_segments_layout_of_the_reference_output(tmp_path):
    from macaw_gb300._lib import RAY_SEGMENT_DTYPE
    # two rays: 3 and 2 segments, chained end to start
    seg = np.zeros(5, RAY_SEGMENT_DTYPE)
    pts = {11: [(0, 0, 0), (1, 0, 0), (1, 1, 0), (1, 1, 1)], 12: [(5, 5, 5), (6, 5, 5), (6, 6, 5)]}
    i = 0
    for rid, p in pts.items():
        for k in range(len(p) - 1):
            seg[i]["id"], seg[i]["segment"], seg[i]["intersections"] = rid, k, k + 1
            seg[i]["start"], seg[i]["end"] = p[k], p[k + 1]
            seg[i]["E"], seg[i]["wgt"], seg[i]["seed_tracking"] = 1e6 - k, 1.0, 2**60 + k
            i += 1
    path = str(tmp_path / "rays.e")
    exodus.write_rays(path, seg, first_history=10)
    with netcdf(path, "r", mmap=False) as f:
        assert _chars(f.variables["name_elem_var"][:]) == REF_RAY_VARS
        assert f.variables["connect1"].elem_type == b"EDGE2"
        assert f.dimensions["num_elem"] == 5 and f.dimensions["num_nodes"] == 5 + 2  # shared nodes per ray
        c = f.variables["connect1"][:] - 1
        x = np.stack([f.variables["coord" + a][:] for a in "xyz"], axis=1)
        assert np.array_equal(x[c[:, 0]], seg["start"]) and np.array_equal(x[c[:, 1]], seg["end"])
        v = {n: f.variables[f"vals_elem_var{k + 1}eb1"][0] for k, n in enumerate(REF_RAY_VARS)}
        assert v["ray_id"].tolist() == [0, 0, 0, 1, 1]
        assert v["aux_id"].tolist() == [11, 11, 11, 12, 12]
        assert v["intersections"].tolist() == [1, 2, 3, 1, 2]
        assert np.array_equal(v["aux_seed_tracking"], seg["seed_tracking"].astype(np.float64))
