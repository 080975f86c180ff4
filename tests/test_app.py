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


@pytest.mark.parametrize("change,message", [
    ("blocks = '0'", "same size as the materials parameter"),
    ("estimator = 'TRACKLENGTH'", "Only the tracklength estimator"),
    ("type = CollisionKernel", "unknown object type"),
    ("scores = 'flux'", "Only the flux score"),
    ("particles = 100000", "must be positive"),
    ("granularity = cell", "Global Tally retrieving currently not supported"),
])
def test_parameter_errors_name_the_parameter(change, message):
    bad = {
        "blocks = '0'": "blocks = '0 1'",
        "estimator = 'TRACKLENGTH'": "estimator = 'COLLISION'",
        "type = CollisionKernel": "type = CollisionKernelX",
        "scores = 'flux'": "scores = 'flux fission'",
        "particles = 100000": "particles = 0",
        "granularity = cell": "granularity = global",
    }[change]
    with pytest.raises(ValueError, match=message):
        app.check_input(CUBE.replace(change, bad))


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
