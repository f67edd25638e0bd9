"""Settings reader (CPU) and the whole-simulation driver fg_run (GPU): the reference's own
functional test (ci-tests/full_test.py) run from its JSON settings through the product's
driver, and the .sol write / restart round trip."""
import json
import os

import numpy as np
import pytest

import feellgood_gb300 as fg

YAML = """# a settings file in the reference's schema
outputs:
  directory: out/     # trailing slash is dropped
  evol_time_step: 2e-13
  final_time: 1e-11
  evol_columns:
    - t
    - <Mx>
    - E_tot
  mag_config_every: false
mesh:
  filename: some/dir/film.msh
  length_unit: 1e-9
  volume_regions:
    film:
      Ae: 1.3e-11
      Ms: 8e5
      K: 1e4
      uk: [0, 0, 2]
      alpha_LLG: 0.02
  surface_regions:
    top: {Ks: 1e-3, suppress_charges: true}
initial_magnetization: [1, 1, 0]
Bext: [0, 0, 0.005]
finite_element_solver:
  max(iter): 500
  tolerance: 1e-8
time_integration:
  max(du): 0.1
  min(dt): 1e-15
  max(dt): 1e-13
"""


def _full_test_settings(golden_dir, outdir, mag_config_every=False):
    g = json.load(open(os.path.join(golden_dir, "golden.json")))["full_test"]
    return g, {
        "outputs": {"directory": str(outdir), "file_basename": "full_test", "evol_time_step": g["evol_time_step"],
                    "final_time": g["final_time"], "mag_config_every": mag_config_every},
        "mesh": {"filename": os.path.join(golden_dir, g["mesh"]), "length_unit": g["length_unit"],
                 "volume_regions": {g["volume_region"]: {"K": g["K"], "uk": g["uk"]}}},
        "initial_magnetization": g["initial_magnetization"],
        "Bext": g["Bext"],
        "time_integration": {"min(dt)": g["min_dt"], "max(dt)": g["max_dt"], "max(du)": g["max_du"]},
    }


def test_settings_yaml(tmp_path):
    p = tmp_path / "s.yml"
    p.write_text(YAML)
    s = fg.settings_dump(p)
    assert s["mesh"] == "some/dir/film.msh" and s["sim_name"] == "film"
    assert s["final_time"] == 1e-11 and s["evol_time_step"] == 2e-13 and s["save_period"] == 0
    assert s["evol_columns"] == ["t", "<Mx>", "E_tot"]
    assert s["tol"] == 1e-8 and s["max_iter"] == 500 and s["dumax"] == 0.1 and s["dt_max"] == 1e-13
    r = s["volume_regions"][0]
    assert r["name"] == "film" and r["Ms"] == 8e5 and r["K"] == 1e4 and r["alpha"] == 0.02
    assert np.allclose(r["uk"], [0, 0, 1])           # unit vectors are normalised
    assert np.allclose(s["m0"], [2 ** -0.5, 2 ** -0.5, 0])
    assert s["Bext"] == [0, 0, 0.005]
    assert s["surface_regions"] == [{"name": "top", "Ks": 1e-3, "suppress_charges": True}]


def test_settings_json_and_defaults(tmp_path, golden_dir):
    g, st = _full_test_settings(golden_dir, tmp_path)
    p = tmp_path / "s.json"
    p.write_text(json.dumps(st))
    s = fg.settings_dump(p)
    assert s["tol"] == 1e-6 and s["max_iter"] == 700     # defaults of the reference
    assert s["volume_regions"][0]["Ms"] == 795774.7 and s["volume_regions"][0]["alpha"] == 0.5
    assert s["volume_regions"][0]["Ae"] == 1e-11
    assert s["evol_columns"] == ["t", "<Mx>", "<My>", "<Mz>", "E_ex", "E_demag", "E_zeeman", "E_tot"]
    assert s["dumax"] == g["max_du"]


def test_settings_errors(tmp_path):
    p = tmp_path / "bad.yml"
    p.write_text("mesh:\n  filename: a.msh\n  volume_regions:\n    v: {Ms: 1}\nBext: [0, 0]\n")
    with pytest.raises(fg.FgError) as e:
        fg.settings_dump(p)
    assert "three components" in str(e.value)
    p.write_text("mesh:\n  filename: a.msh\n  volume_regions:\n    v: {Ms: 1}\ninitial_magnetization: [sin(x), 0, 1]\n")
    with pytest.raises(fg.FgError):
        fg.settings_dump(p)
    for key in ("solver_threads", "solver_blocks", "checkpoint_every"):  # counts >= 0
        p.write_text("mesh:\n  filename: a.msh\n  volume_regions:\n    v: {Ms: 1}\ngpu: {%s: -1}\n" % key)
        with pytest.raises(fg.FgError) as e:
            fg.settings_dump(p)
        assert key in str(e.value)


def _last_row(path):
    rows = [l for l in open(path) if not l.startswith("#")]
    return np.array([float(x) for x in rows[-1].split()])


@pytest.mark.gpu
def test_run_full_test_golden(tmp_path, golden_dir):
    g, st = _full_test_settings(golden_dir, tmp_path)
    p = tmp_path / "full_test.json"
    p.write_text(json.dumps(st))
    rep = fg.run(p, seed=g["seed"])
    assert rep["steps"] > 0 and abs(rep["t"] - g["final_time"]) < 1e-20
    last = _last_row(tmp_path / "full_test.evol")
    exp = g["expected_5pt"]
    assert np.linalg.norm(last[1:4] - np.array(exp["m"])) < g["threshold"]
    assert abs((last[7] - exp["E_tot"]) / exp["E_tot"]) < g["threshold"]
    hdr = [l for l in open(tmp_path / "full_test.evol") if l.startswith("## columns:")][0]
    assert hdr.split(":", 1)[1].split() == ["t", "<Mx>", "<My>", "<Mz>", "E_ex", "E_demag", "E_zeeman", "E_tot"]


@pytest.mark.gpu
def test_sol_written_and_restarted(tmp_path, golden_dir):
    g, st = _full_test_settings(golden_dir, tmp_path, mag_config_every=5)
    st["outputs"]["final_time"] = 5e-12
    p = tmp_path / "a.json"
    p.write_text(json.dumps(st))
    fg.run(p, seed=1)
    sol = tmp_path / "full_test_iter5.sol"
    text = open(sol).read().splitlines()
    assert any(l.startswith("## time: ") for l in text)
    data = np.array([[float(x) for x in l.split()] for l in text if not l.startswith("#")])
    assert data.shape[1] == 5 and np.array_equal(data[:, 0], np.arange(len(data)))
    assert np.allclose(np.linalg.norm(data[:, 1:4], axis=1), 1.0, atol=1e-6)
    # restart from the snapshot: time is taken from its metadata
    st2 = dict(st)
    st2["initial_magnetization"] = str(sol)
    st2["outputs"] = dict(st["outputs"], file_basename="restart", final_time=6e-12, mag_config_every=False)
    p2 = tmp_path / "b.json"
    p2.write_text(json.dumps(st2))
    rep = fg.run(p2, seed=1)
    assert abs(rep["t"] - 6e-12) < 1e-20
    first = [l for l in open(tmp_path / "restart.evol") if not l.startswith("#")][0].split()
    assert abs(float(first[0]) - 5e-12) < 1e-20


@pytest.mark.gpu
@pytest.mark.parametrize("gpu", [{}, {"precision": "fp32_refine", "demag": "fmm"}])
def test_checkpoint_resume_is_bitwise(tmp_path, golden_dir, gpu):
    """A run stopped at a full-precision checkpoint (gpu.checkpoint_every) and resumed from
    it (gpu.resume) writes the same .evol rows, to the last printed digit (%.16g), as the
    uninterrupted run: the checkpoint keeps u, v, phi, phiv in FP64, the step controller, the
    basis-angle stream position and the solver / FMM choices that fix the arithmetic order
    (the uninterrupted run is given the choices the first half timed)."""
    g, st = _full_test_settings(golden_dir, tmp_path)
    total = 12 * g["evol_time_step"]
    cols = ["t", "<Mx>", "<My>", "<Mz>", "E_ex", "E_demag", "E_zeeman", "E_tot"]
    # first half, checkpoint after row 6 (rows 0..6 = 7 rows)
    half = dict(st, gpu=dict(gpu, checkpoint_every=7),
                outputs=dict(st["outputs"], file_basename="split", final_time=6 * g["evol_time_step"],
                             evol_columns=cols))
    (tmp_path / "half.json").write_text(json.dumps(half))
    fg.run(tmp_path / "half.json", seed=3)
    ck = tmp_path / "split.ckpt"
    head = fg.checkpoint_peek(ck)
    assert head["output_index"] == 7 and head["rng_seed"] == 3 and head["steps"] > 0
    rest = dict(half, gpu=dict(gpu, resume=str(ck)), outputs=dict(half["outputs"], final_time=total))
    (tmp_path / "rest.json").write_text(json.dumps(rest))
    rep = fg.run(tmp_path / "rest.json", seed=12345)  # the checkpoint's seed and stream position win
    assert abs(rep["t"] - total) < 1e-20
    fixed = dict(solver_lanes_per_row=head["solver_lpr"], solver_blocks=head["solver_blocks"],
                 solver_threads=head["solver_threads"], fmm_depth=head["fmm_depth"])
    full = dict(st, gpu=dict(gpu, **fixed), outputs=dict(st["outputs"], file_basename="full", final_time=total,
                                                        evol_columns=cols))
    (tmp_path / "full.json").write_text(json.dumps(full))
    fg.run(tmp_path / "full.json", seed=3)
    a = [l for l in open(tmp_path / "full.evol") if not l.startswith("#")]
    b = [l for l in open(tmp_path / "split.evol") if not l.startswith("#")]
    assert len(a) == len(b) == 13
    assert a == b


SPIN_YAML = """
outputs: {directory: out, final_time: 1e-12}
mesh:
  filename: wire.msh
  volume_regions:
    cu: {Ms: 0, sigma: 5.8e7, dens_state: 1e47, P: 0, l_sf: 300e-9}
    py: {sigma: 5e6, dens_state: 1e47, P: 0.5, l_sd: 1e-9, l_sf: 5e-9}
  surface_regions:
    ground: {V: 0, s: [0, 0, 0]}
    contact: {jn: 1e11, uP: [0, 2, 0]}
spin_accumulation: {enable: true, V_file: true}
recentering: {enable: true, direction: Y, threshold: 0.2}
"""


def test_settings_spin_accumulation(tmp_path):
    """spin_accumulation and the regions' spin parameters and boundary conditions are read
    with the reference's keys (src/default-settings.yml)."""
    p = tmp_path / "spin.yml"
    p.write_text(SPIN_YAML)
    s = fg.settings_dump(p)["spin_accumulation"]
    assert s["enable"] and s["V_file"]
    vol = {r["name"]: r for r in s["volume"]}
    assert vol["cu"]["sigma"] == 5.8e7 and vol["cu"]["l_sf"] == 300e-9 and vol["py"]["l_sd"] == 1e-9
    assert vol["py"]["P"] == 0.5 and vol["py"]["dens_state"] == 1e47
    surf = {r["name"]: r for r in s["surface"]}
    assert surf["ground"]["V"] == 0 and surf["ground"]["s"] == [0, 0, 0] and surf["ground"]["jn"] is None
    assert surf["contact"]["jn"] == 1e11 and surf["contact"]["uP"] == [0, 1, 0] and surf["contact"]["V"] is None
    assert fg.settings_dump(p)["recentering"] == {"enable": True, "direction": 1, "threshold": 0.2}
