"""Input-file front end (MaCaw HIT blocks -> C ABI)."""
import numpy as np
import pytest

from macaw_gb300 import app

CUBE = app.read("cube.i")


def test_bundled_inputs_check():
    c = app.check_input(CUBE)
    assert c["tets"] == 48000 and c["nuclides"] == 10 and c["materials"] == 1 and c["particles"] == 100000
    lat = app.check_input(app.read("lattice.i"))
    assert lat["tets"] == 2039184 and lat["nuclides"] == 22 and lat["batches"] == 10 and lat["aux"] == 2


def test_reflective_bcs_and_paths():
    txt = CUBE.replace("type = KillRayBC", "type = ReflectRayBC")
    assert app.check_input(txt)["reflective"] == 6
    # an [a/b] path header is the same as nested blocks
    nested = "[RayBCs]\n  [vacuum]\n    type = ReflectRayBC\n    boundary = 'back front top right left bottom'\n  []\n[]"
    assert nested in txt
    path = "[RayBCs/vacuum]\n  type = ReflectRayBC\n  boundary = 'back front top right left bottom'\n[]"
    assert app.check_input(txt.replace(nested, path))["reflective"] == 6


@pytest.mark.parametrize("change,bad,message", [
    ("blocks = '0'", "blocks = '0 1'", "same size as the materials parameter"),
    ("estimator = 'TRACKLENGTH'", "estimator = 'ANALOG'", "analog estimator is not available"),
    ("type = CollisionKernel", "type = CollisionKernelX", "unknown object type"),
    ("scores = 'flux'", "scores = 'flux fission'", "score 'fission' is not available"),
    ("scores = 'flux'", "scores = 'flux scatter'", "scores flux and total only"),
    ("filters = 'cell'", "filters = 'cell energy'", "energy bins parameter should be supplied"),
    ("filters = 'cell'", "filters = 'mesh'", "unknown filter"),
    ("score = 'flux'", "score = 'total'", "score does not exist in given tally"),
    ("particles = 100000", "particles = 0", "must be positive"),
    ("granularity = cell", "granularity = global", "Global Tally retrieving currently not supported"),
])
def test_parameter_errors_name_the_parameter(change, bad, message):
    assert change in CUBE
    with pytest.raises(ValueError, match=message):
        app.check_input(CUBE.replace(change, bad))


# a tally block as the reference's own inputs write it (test/tests/tally/openmc_tally.i,
# test/tests/assembly/run_assembly.i): collision estimator, several scores, energy filter
REF_STYLE = CUBE.replace("estimator = 'TRACKLENGTH'\n    scores = 'flux'\n    filters = 'cell'",
                         "estimator = 'COLLISION'\n    scores = 'flux scatter absorption'\n"
                         "    filters = 'energy particle cell'\n    energy_bins = '1e-5 1e3 2e7'").replace(
    "estimator = TRACKLENGTH", "estimator = COLLISION")


def test_reference_style_collision_tally_checks():
    assert "COLLISION" in REF_STYLE and "energy_bins" in REF_STYLE
    c = app.check_input(REF_STYLE)
    assert c["tally_values_per_element"] == 2 * 3
    one_bin = REF_STYLE.replace("score = 'flux'", "score = 'scatter'\n    energy_bin = 1")
    assert app.check_input(one_bin)["aux"] == 1
    with pytest.raises(ValueError, match="energy bin"):
        app.check_input(REF_STYLE.replace("score = 'flux'", "score = 'flux'\n    energy_bin = 2"))


def test_unused_parameter_and_syntax_errors():
    with pytest.raises(ValueError, match="unused parameter"):
        app.check_input(CUBE.replace("blocks = '0'", "blocks = '0'\n  colour = blue"))
    with pytest.raises(ValueError, match="unterminated"):
        app.check_input(CUBE + "\n[Extra]\n  a = 1\n")
    with pytest.raises(ValueError, match="missing required parameter"):
        app.check_input(CUBE.replace("  temperature = temperature\n", ""))


@pytest.mark.gpu
def test_run_matches_direct_api(tmp_path):
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_TALLY_SUM
    txt = CUBE.replace("particles = 100000", "particles = 20000").replace("num_steps = 1", "num_steps = 2")
    txt = txt.replace("csv = true", "csv = true\n  exodus = true")
    assert "exodus = true" in txt
    rep = app.run_input(txt, 0, str(tmp_path / "cube"))
    assert rep["histories"] == 40000 and rep["stuck"] == 0 and rep["lost"] == 0
    csv = np.loadtxt(tmp_path / "cube_flux.csv", delimiter=",", skiprows=1)
    p = problems.cube_problem()
    with Tracker(0) as t:
        t.load(p)
        for b in range(2):
            t.run(20000, first=20000 * b, seed=1, accumulate=True)
        ref = t.tally(MC_TALLY_SUM) / 2
    got = csv[:, 2]
    nz = ref > 0
    assert np.all(np.abs(got[nz] - ref[nz]) <= 1e-12 * ref[nz])
    assert rep["aux"]["flux"]["sum"] == pytest.approx(2 * ref.sum(), rel=1e-12)
    # the same field in the Exodus output (one block: the cube's subdomain 0)
    from scipy.io import netcdf_file
    with netcdf_file(rep["exodus"], "r", mmap=False) as f:
        assert np.array_equal(f.variables["vals_elem_var1eb1"][0], got)


@pytest.mark.gpu
def test_reference_style_collision_tally_runs(tmp_path):
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_EST_COLLISION, MC_SCORE_ABSORPTION, MC_SCORE_FLUX, MC_SCORE_SCATTER, MC_TALLY_SUM
    txt = REF_STYLE.replace("particles = 100000", "particles = 20000").replace(
        "score = 'flux'", "score = 'scatter'")
    rep = app.run_input(txt, 0, str(tmp_path / "cube"))
    assert rep["histories"] == 20000 and rep["collisions"] > 0
    p = problems.cube_problem()
    p.tally = problems.TallyDef(MC_EST_COLLISION, (MC_SCORE_FLUX, MC_SCORE_SCATTER, MC_SCORE_ABSORPTION),
                                np.array([1e-5, 1e3, 2e7]))
    with Tracker(0) as t:
        t.load(p)
        t.run(20000, seed=1, accumulate=True)
        ref = t.tally(MC_TALLY_SUM).reshape(p.n_tet, 2, 3)[:, :, 1].sum(axis=1)  # scatter, both bins
    csv = np.loadtxt(tmp_path / "cube_flux.csv", delimiter=",", skiprows=1)
    nz = ref > 0
    assert np.all(np.abs(csv[nz, 2] - ref[nz]) <= 1e-12 * ref[nz])


def test_file_mesh_generator_reads_an_exodus_tet_mesh(tmp_path, monkeypatch):
    from macaw_gb300 import exodus, problems
    p = problems.cube_problem()
    exodus.write(str(tmp_path / "cube_mesh.e"), p, {})
    monkeypatch.chdir(tmp_path)
    start, end = CUBE.index("[Mesh]"), CUBE.index("[]\n[]", CUBE.index("[Mesh]")) + 5
    txt = CUBE[:start] + "[Mesh]\n  [fmg]\n    type = FileMeshGenerator\n    file = 'cube_mesh.e'\n  []\n[]\n" + CUBE[end:]
    c = app.check_input(txt)
    assert c["tets"] == p.n_tet and c["vertices"] == p.xyz.shape[0]
    with pytest.raises(ValueError, match="file"):
        app.check_input(txt.replace("cube_mesh.e", "missing.e"))


@pytest.mark.gpu
def test_ray_tracing_exodus_output(tmp_path):
    from scipy.io import netcdf_file
    txt = CUBE.replace("particles = 100000", "particles = 2000").replace(
        "csv = true", "csv = true\n  [rays]\n    type = RayTracingExodus\n    study = study\n    output_data = true\n"
                      "    output_aux_data = true\n    execute_on = final\n    max_rays = 30\n  []")
    rep = app.run_input(txt, 0, str(tmp_path / "cube"))
    assert rep["rays"].endswith("cube_rays.e") and rep["ray_segments"] > 30
    with netcdf_file(rep["rays"], "r", mmap=False) as f:
        assert f.dimensions["num_elem"] == rep["ray_segments"]
        ray_id = f.variables["vals_elem_var10eb1"][0]
        assert set(np.unique(ray_id).astype(int)) == set(range(30))


def _lattice_2d_input():
    txt = app.read("lattice.i")
    txt = txt.replace("nz = 21", "nz = 1").replace("height = 50", "height = 1")
    txt = txt.replace("materials = '1 2 3'\n[]", "materials = '1 2 3'\n  z_coord = 0.5\n[]")
    txt = txt.replace("boundary = 'back front top right left bottom'",
                      "boundary = 'top right left bottom'\n  []\n  [planes]\n    type = ReflectRayBC\n"
                      "    boundary = 'back front'")
    return txt.replace("particles = 1000000", "particles = 20000").replace("num_steps = 10", "num_steps = 1")


def test_two_d_input_checks():
    txt = _lattice_2d_input()
    assert "z_coord = 0.5" in txt and "ReflectRayBC" in txt
    c = app.check_input(txt)
    assert c["tets"] == 2039184 // 21 and c["reflective"] == 2


@pytest.mark.gpu
def test_two_d_input_runs_like_the_direct_api(tmp_path):
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_TALLY_SUM
    rep = app.run_input(_lattice_2d_input(), 0, str(tmp_path / "l2d"))
    assert rep["histories"] == 20000 and rep["stuck"] == 0
    p = problems.lattice_2d_problem()
    with Tracker(0) as t:
        t.load(p)
        t.run(20000, seed=1, accumulate=True, bank_size=1000000)
        ref = t.tally(MC_TALLY_SUM)
    assert rep["aux"]["flux"]["sum"] == pytest.approx(ref.sum(), rel=1e-12)


def _small_eigen_input():
    txt = app.read("eigen_lattice.i")
    for a, b in (("nx = 17", "nx = 5"), ("ny = 17", "ny = 5"), ("nz = 21", "nz = 6"), ("height = 50", "height = 15"),
                 ("n_points = 20000", "n_points = 3000"), ("particles = 1000000", "particles = 5000"),
                 ("bank_size = 1000000", "bank_size = 2048"), ("inactive = 3", "inactive = 2"),
                 ("num_steps = 13", "num_steps = 4")):
        assert a in txt
        txt = txt.replace(a, b)
    return txt


def test_eigen_input_checks():
    c = app.check_input(app.read("eigen_lattice.i"))
    assert c["run_mode"] == "eigenvalue" and c["inactive"] == 3 and c["fissionable_nuclides"] == 15
    assert c["tets"] == 2039184 and c["reflective"] == 4 and c["batches"] == 13
    with pytest.raises(ValueError, match="inactive batches need run_mode"):
        app.check_input(app.read("lattice.i").replace("precision = fp64", "precision = fp64\n    inactive = 2"))
    with pytest.raises(ValueError, match="not in material_ids"):
        app.check_input(app.read("eigen_lattice.i").replace("fissionable_materials = '1'", "fissionable_materials = '7'"))


@pytest.mark.gpu
def test_eigen_input_runs_like_the_direct_api(tmp_path):
    from macaw_gb300 import Tracker, problems
    from macaw_gb300._lib import MC_TALLY_SUM
    rep = app.run_input(_small_eigen_input(), 0, str(tmp_path / "eig"))
    p = problems.eigen_lattice_problem(nx=5, ny=5, nz=6, height=15.0, n_pts=3000)
    with Tracker(0) as t:
        t.load(p)
        g = t.eigen(5000, 4, 2, seed=1, bank_size=2048)
        ref = t.tally(MC_TALLY_SUM) / 2
    assert [x["k_generation"] for x in rep["generations"]] == list(g["k_generation"])
    assert rep["keff"] == g["keff"][-1] and rep["keff_std"] == g["keff_std"][-1]
    k = np.loadtxt(tmp_path / "eig_keff.csv", delimiter=",", skiprows=1)
    assert np.array_equal(k[:, 2], g["keff"])
    csv = np.loadtxt(tmp_path / "eig_flux.csv", delimiter=",", skiprows=1)
    nz = ref > 0
    assert np.all(np.abs(csv[nz, 2] - ref[nz]) <= 1e-12 * ref[nz])


def test_command_line_check(capsys):
    """python -m macaw_gb300.app INPUT --check prints the validated summary."""
    import json
    from macaw_gb300 import app
    from macaw_gb300.app import INPUTS
    assert app.main([str(INPUTS / "eigen_lattice.i"), "--check"]) == 0
    rep = json.loads(capsys.readouterr().out)
    assert rep["tets"] == 2039184 and rep["run_mode"] == "eigenvalue"
