"""The oracle's restatement of the reference's output writers (oracle/rbtp_oracle_io.c) on fixed
values: the printf formats of statistics.dat (output_statis.cu:102-106), Nu_%.2e.txt
(output_statis.cu:216-219), Profile_%.2e.txt (output_statis.cu:238-282) and pos/pos_%09d.txt
(output_part.cu:91-115), the raw-double layouts of %09d.dat and fg%09d.dat (output_flow.cu:64-127)
with the solid-node overwrite, and the output directory name (output_statis.cu:66)."""
import numpy as np

from rbtp import workloads as W


def test_text_formats(oracle_mod, tmp_path):
    d = str(tmp_path)
    assert oracle_mod.output_dirname(1e6, 0.71) == "Ra1.0e+06Pr0.71"
    oracle_mod.write_statistics(d, 10, [1e-3, -2e-19, 3.0, 0.5])
    oracle_mod.write_statistics(d, 125, [0.0, 1.0, -1.0, 0.25])
    assert (tmp_path / "statistics.dat").read_text() == (
        "10        1.000000e-03  -2.000000e-19   3.000000e+00   5.000000e-01\n"
        "125       0.000000e+00   1.000000e+00  -1.000000e+00   2.500000e-01\n")
    oracle_mod.write_nu(d, 1e6, (10, 0.04, 1.23, 1.1, 1.2, 1.0, 0.2))
    assert (tmp_path / "Nu_1.00e+06.txt").read_text() == (
        "   1.000000E+01   4.000000E-02   1.230000E+00   1.100000E+00   1.200000E+00   1.000000E+00"
        "   2.000000E-01\n")
    oracle_mod.write_profile(d, 1e6, 7, np.arange(8.0).reshape(2, 4))
    assert (tmp_path / "Profile_1.00e+06.txt").read_text() == (
        "7\n  0.000000e+00   1.000000e+00   2.000000e+00   3.000000e+00\n"
        "  4.000000e+00   5.000000e+00   6.000000e+00   7.000000e+00\n")
    oracle_mod.write_particles(d, 3, np.arange(66.0).reshape(2, 33))
    lines = (tmp_path / "pos" / "pos_000000003.txt").read_text().split("\n")
    assert lines[0] == "0 " + " ".join(f"{v:14.6e}" for v in range(33))
    assert lines[1] == "1 " + " ".join(f"{v:14.6e}" for v in range(33, 66)) and lines[2] == ""


def test_binary_layouts_and_solid_overwrite(oracle_mod, tmp_path):
    cfg = W.config("plain_fp64", lx=4, ly=3, lz=2)
    L = cfg.nodes
    fields = np.arange(7 * L, dtype=np.float64) + 0.5
    owner = -np.ones(L, dtype=np.int32)
    owner[5] = 0                                   # node (x, y, z) = (1, 1, 0) belongs to sphere 0
    row = np.zeros((1, 33))
    row[0, :3] = (1.2, 1.4, 0.6)
    row[0, 3:6] = (0.1, 0.2, 0.3)
    row[0, 18:21] = (0.01, 0.02, 0.03)
    row[0, 30] = 0.75
    oracle_mod.write_flow(str(tmp_path), 40, cfg, fields, owner, row)
    got = np.fromfile(tmp_path / "000000040.dat").reshape(7, L)
    want = fields.reshape(7, L).copy()
    rel = np.array([1.5 - 1.2, 1.5 - 1.4, 0.5 - 0.6])
    w, v = row[0, 18:21], row[0, 3:6]
    want[:, 5] = [cfg.rho0, v[0] + (rel[2] * w[1] - rel[1] * w[2]), v[1] + (rel[0] * w[2] - rel[2] * w[0]),
                  v[2] + (rel[1] * w[0] - rel[0] * w[1]), 0.75, 0.0, 0.0]
    assert np.array_equal(got, want)
    f, g = np.arange(27 * L, dtype=np.float64), -np.arange(27 * L, dtype=np.float64)
    oracle_mod.write_fg(str(tmp_path), 40, f, g)
    assert np.array_equal(np.fromfile(tmp_path / "fg000000040.dat"), np.concatenate([f, g]))
