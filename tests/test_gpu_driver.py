"""Config-driven runner (navier-stokes-solvers_gb300/ns_run): INI then JSON override
(the reference's config layering, config_parser.c:543-554), Taylor-Green decay,
spectrum and checkpoint files, and configuration errors."""
import json
import math
import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUNNER = os.path.join(ROOT, "navier-stokes-solvers_gb300", "ns_run")


def _run(tmp_path, ini: str, override: dict | None = None):
    p = tmp_path / "params.ini"
    p.write_text(ini)
    args = [RUNNER, str(p)]
    if override is not None:
        o = tmp_path / "override.json"
        o.write_text(json.dumps(override))
        args.append(str(o))
    return subprocess.run(args, capture_output=True, text=True, timeout=120)


def _lines(stdout):
    rows = []
    for line in stdout.splitlines():
        tok = line.split()
        if tok and tok[0] == "step":
            rows.append({tok[i]: float(tok[i + 1]) for i in range(0, len(tok), 2)})
    return rows


def test_taylor_green_decay_with_overrides(nsgb, tmp_path):
    ini = f"""[solver]
type = spectral
[grid]
nx = 32
ny = 32
[fluid]
Re = 1000.0
[time]
dt = 0.01
t_end = 0.5
[output]
dir = {tmp_path}
every = 10
spectrum_every = 25
checkpoint_every = 50
"""
    # JSON overrides the INI viscosity (Re 1000 -> 100), as the reference's layering does
    r = _run(tmp_path, ini, {"fluid": {"Re": 100.0}})
    assert r.returncode == 0, r.stderr
    rows = _lines(r.stdout)
    assert rows[0]["step"] == 0 and rows[-1]["t"] >= 0.5 - 1e-12
    # the reference Taylor-Green state has |k|^2 = 2: energy decays as exp(-4 t / Re)
    for row in rows:
        assert abs(row["energy"] / rows[0]["energy"] - math.exp(-4.0 * row["t"] / 100.0)) <= 1e-6
    assert (tmp_path / "spectrum_000025.dat").exists() and (tmp_path / "solution.dat").exists()
    z = np.load(tmp_path / "checkpoint_000050.npz")
    assert int(z["nx"]) == 32 and abs(float(z["Re"]) - 100.0) < 1e-12 and abs(float(z["time"]) - 0.5) < 1e-9
    spec = np.loadtxt(tmp_path / "spectrum_000025.dat")
    assert spec.shape[1] == 4 and spec[1, 1] > 0  # the |k| = 1.41 shell holds the energy


def test_forced_random_run_fp32(nsgb, tmp_path):
    ini = f"""[grid]
nx = 64
ny = 64
[fluid]
Re = 10000.0
[time]
cfl = 0.5
t_end = 100.0
steps = 40
[spectral]
precision = fp32
[spectral.hyperviscosity]
coefficient = 5.0
order = 4
cutoff_ratio = 0.0
[ic]
type = random
seed = 3
k0 = 4.0
[forcing]
type = white
epsilon = 0.001
[output]
dir = {tmp_path}
every = 20
solution = 0
"""
    r = _run(tmp_path, ini)
    assert r.returncode == 0, r.stderr
    rows = _lines(r.stdout)
    assert [int(x["step"]) for x in rows] == [0, 20, 40]
    assert all(np.isfinite(x["energy"]) and 0.2 < x["energy"] < 0.8 for x in rows)
    assert not (tmp_path / "solution.dat").exists()


def test_vtk_snapshots_written_asynchronously(nsgb, tmp_path):
    """output.vtk_every: legacy VTK files (the reference's structured-grid layout)
    of the device state, written by a writer thread while the solver continues;
    the last one holds the same fields as the final solution.dat."""
    ini = f"""[grid]
nx = 32
ny = 16
[fluid]
Re = 100.0
[time]
dt = 0.01
t_end = 100.0
steps = 50
[output]
dir = {tmp_path}
every = 10
vtk_every = 25
"""
    r = _run(tmp_path, ini)
    assert r.returncode == 0, r.stderr
    rows = _lines(r.stdout)
    assert [int(x["step"]) for x in rows][-1] == 50
    for step in (25, 50):
        assert (tmp_path / f"solution_{step:06d}.vtk").exists()
    lines = (tmp_path / "solution_000050.vtk").read_text().splitlines()
    assert lines[0] == "# vtk DataFile Version 3.0" and lines[3] == "DATASET STRUCTURED_GRID"
    assert lines[4] == "DIMENSIONS 32 16 1" and lines[5] == "POINTS 512 double"
    n = 512
    t_line = lines[6 + n + 2]
    assert abs(float(t_line) - rows[-1]["t"]) < 1e-9
    i_vec = lines.index("VECTORS velocity double")
    uv = np.array([[float(a) for a in ln.split()[:2]] for ln in lines[i_vec + 1:i_vec + 1 + n]])
    i_sc = lines.index("SCALARS vorticity double 1")
    w = np.array([float(a) for a in lines[i_sc + 2:i_sc + 2 + n]])
    sol = np.loadtxt(tmp_path / "solution.dat")  # x y u v omega psi at the end
    assert np.abs(uv[:, 0] - sol[:, 2]).max() < 1e-8 and np.abs(uv[:, 1] - sol[:, 3]).max() < 1e-8
    assert np.abs(w - sol[:, 4]).max() < 1e-8


def test_configuration_errors(nsgb, tmp_path):
    r = _run(tmp_path, "[grid]\nnx = 32\n")  # grid.ny and fluid.Re are required
    assert r.returncode == 2 and "ny" in r.stderr
    r = _run(tmp_path, "[grid]\nnx = 32\nny = 32\n[fluid]\nRe = 10\n[spectral]\nprecision = fp16\n")
    assert r.returncode == 2
