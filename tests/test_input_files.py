"""Input files of the input-file Lanczos program: the writer reproduces the
reference's prepare_input_files byte for byte (tests/golden/
input_files_m6_n5_s48.npz holds the text the reference wrote)."""
import os

import numpy as np

from tdscha_gb300.DynamicalLanczos import Lanczos


def _split_syms(d):
    M = len(d["w"])
    S = int(d["S"])
    syms, spaces, o_s, o_d = [], [], 0, 0
    for n in d["n_deg"]:
        syms.append(d["sym"][o_s:o_s + S * n * n].reshape(S, n, n))
        spaces.append(d["deg_space"][o_d:o_d + n])
        o_s += S * n * n
        o_d += n
    assert o_d == M
    return syms, spaces


def test_prepare_input_files_matches_reference_text(golden, tmp_path):
    d = golden("input_files_m6_n5_s48.npz")
    lz = Lanczos.from_arrays(d["X"], d["Y"], d["w"], d["rho"], float(d["T"]), use_wigner=False)
    lz.init(symmetries=_split_syms(d))
    lz.psi = d["psi"].copy()
    lz.perturbation_modulus = float(d["psi"][:6].dot(d["psi"][:6]))
    lz.prepare_input_files(root_name="case", n_steps=7, directory=str(tmp_path))
    written = sorted(os.listdir(tmp_path))
    expected = sorted(k[len("file:"):] for k in d if k.startswith("file:"))
    assert [w[len("case"):] for w in written] == expected
    for suffix in expected:
        with open(tmp_path / ("case" + suffix)) as fp:
            assert fp.read() == str(d["file:" + suffix]), suffix


def test_load_from_input_files(tmp_path):
    lz = Lanczos.from_arrays(np.zeros((3, 2)), np.zeros((3, 2)), [0.01, 0.02], np.ones(3), 300.0)
    lz.init(use_symmetries=False)
    lz.prepare_input_files("r", n_steps=3, directory=str(tmp_path))
    with open(tmp_path / "r.abc", "w") as fp:
        fp.write("1.0e-6\t2.0e-7\t2.1e-7\n3.0e-6\t4.0e-7\t4.1e-7\n5.0e-6\n")
    P = 2 + 2 * 3
    np.savetxt(tmp_path / "r.qbasis.out", np.ones((3, P)))
    np.savetxt(tmp_path / "r.pbasis.out", 2 * np.ones((3, P)))
    np.savetxt(tmp_path / "r.snorm.out", [1.0, 0.5, 0.25])
    lz2 = Lanczos()
    lz2.load_from_input_files("r", directory=str(tmp_path))
    assert lz2.a_coeffs == [1e-6, 3e-6, 5e-6]
    assert lz2.b_coeffs == [2e-7, 4e-7] and lz2.c_coeffs == [2.1e-7, 4.1e-7]
    assert lz2.s_norm == [1.0, 0.5, 0.25]
    assert lz2.n_modes == 2 and lz2.N == 3 and lz2.T == 300.0
