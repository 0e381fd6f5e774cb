"""The input-file Lanczos program (tdscha-lanczos-gb300) end to end against the
reference's own bi-Lanczos run (tests/golden/runft_m21_n1000.npz)."""
import json
import os
import subprocess

import numpy as np
import pytest

from tdscha_gb300 import build
from tdscha_gb300.DynamicalLanczos import Lanczos

pytestmark = pytest.mark.gpu


def _run(root, *extra):
    r = subprocess.run([build.EXE, root] + list(extra), capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    return r


def _prepare(d, directory, n_steps):
    lz = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=False)
    lz.init(use_symmetries=False)
    lz.psi[:] = 0
    lz.psi[:len(d["R1"])] = d["R1"]
    lz.perturbation_modulus = float(d["R1"].dot(d["R1"]))
    lz.prepare_input_files("run", n_steps=n_steps, directory=directory)
    return os.path.join(directory, "run")


def test_executable_matches_reference_bilanczos(gpu_lib, golden, tmp_path):
    d = golden("runft_m21_n1000.npz")
    root = _prepare(d, str(tmp_path), 50)
    _run(root)
    lz = Lanczos()
    lz.load_from_input_files("run", directory=str(tmp_path))
    for t in "abc":
        np.testing.assert_allclose(getattr(lz, t + "_coeffs"), d["bilanczos/" + t], rtol=1e-8)
    assert len(lz.s_norm) == 51
    Q = np.loadtxt(str(tmp_path / "run.qbasis.out"))
    assert Q.shape == (51, 21 + 21 * 22)


def test_executable_restart(gpu_lib, golden, tmp_path):
    d = golden("runft_m21_n1000.npz")
    root = _prepare(d, str(tmp_path), 20)
    _run(root, "--chunk", "7")
    with open(root + ".json") as fp:
        js = json.load(fp)
    js.update(n_steps=35, restart=True, step_done=20)
    with open(root + ".json", "w") as fp:
        json.dump(js, fp)
    _run(root)
    lz = Lanczos()
    lz.load_from_input_files("run", directory=str(tmp_path))
    np.testing.assert_allclose(lz.a_coeffs, d["bilanczos/a"][:35], rtol=1e-8)
    np.testing.assert_allclose(lz.b_coeffs, d["bilanczos/b"][:35], rtol=1e-8)
