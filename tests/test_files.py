"""The file formats of the reference's examples/tools/savetools.jl and the
checkpoint file.  The CPU tests cover the number format (Julia's print of a
Float64) and the density table; the GPU tests write the paths table from the
device state and round-trip a checkpoint."""
import os

import numpy as np
import pytest


def test_numbers_print_as_julia_prints_them(engine_lib):
    from pimc.engine import julia_float
    cases = [(0.5, "0.5"), (1e-5, "1.0e-5"), (0.0001, "0.0001"), (1234567.0, "1.234567e6"),
             (123456.0, "123456.0"), (1e6, "1.0e6"), (-2.5, "-2.5"),
             (0.1 + 0.2, "0.30000000000000004"), (5e-324, "5.0e-324"),
             (1.7976931348623157e308, "1.7976931348623157e308"), (0.0, "0.0"), (-0.0, "-0.0"),
             (float("inf"), "Inf"), (float("-inf"), "-Inf"), (12.0, "12.0"),
             (6.666666666666667e-05, "6.666666666666667e-5"), (-0.000123, "-0.000123")]
    for x, want in cases:
        assert julia_float(x) == want, (x, julia_float(x), want)
    assert julia_float(float("nan")) == "NaN"
    rng = np.random.default_rng(1)
    for x in rng.standard_normal(200) * 10.0 ** rng.integers(-8, 9, 200):
        assert float(julia_float(float(x))) == x  # round trip


def test_density_table_layout(engine_lib, tmp_path):
    from pimc.engine import write_density_csv
    nb, L, nd = 4, 2.0, 10
    counts = np.arange(nb * nb, dtype=float).reshape(nb, nb, order="F")  # counts[i, k]
    p = tmp_path / "d.csv"
    write_density_csv(str(p), 2, nb, L, counts, nd)
    lines = p.read_text().splitlines()
    assert lines[0] == "pos,x1,x2,x3,x4"
    assert [l.split(",")[0] for l in lines[1:]] == ["-2.0", "-0.6666666666666666",
                                                    "0.6666666666666666", "2.0"]
    tab = np.array([[float(v) for v in l.split(",")[1:]] for l in lines[1:]])
    np.testing.assert_array_equal(tab, counts / ((2 * L / nb) * nd))
    write_density_csv(str(p), 1, 3, 1.5, np.array([3.0, 0.0, 6.0]), 3)
    assert p.read_text().splitlines() == ["pos,Density", "-1.5,1.0", "0.0,0.0", "1.5,2.0"]


def test_density_file_name_follows_the_reference(engine_lib):
    from types import SimpleNamespace

    from pimc.api import density_filename
    s = SimpleNamespace(M=200, β=1 / 0.2, N=20)
    assert density_filename(s, 2.0, "l25", 4.0) == "densityl25M200beta5.0N20g2.0V4.0.csv"


@pytest.mark.gpu
def test_paths_table_from_the_device(engine_lib, tmp_path):
    from pimc.engine import ChainParams, Engine
    N, M, L = 3, 4, 3.0
    e = Engine(ChainParams(dim=2, N=N, M=M, L=L, T=2.0, lam=0.5))
    rng = np.random.default_rng(3)
    x = rng.uniform(-L, L, size=(2, N, M))
    nxt = np.array([1, 2, 0], dtype=np.int32)
    e.set_beads(x)
    e.set_next(nxt)
    p = tmp_path / "paths.csv"
    e.write_paths_csv(str(p))
    lines = p.read_text().splitlines()
    assert lines[0] == "tau,p1 x,p1 y,p2 x,p2 y,p3 x,p3 y"
    assert len(lines) == M + 2
    tab = np.array([[float(v) for v in l.split(",")] for l in lines[1:]])
    np.testing.assert_array_equal(tab[:, 0], [j * 0.5 / M for j in range(M + 1)])
    for n in range(N):
        for d in range(2):
            col = tab[:, 1 + 2 * n + d]
            np.testing.assert_array_equal(col[:M], x[d, n])
            assert col[M] == x[d, nxt[n], 0]


@pytest.mark.gpu
def test_checkpoint_file_round_trip(engine_lib, tmp_path):
    from pimc import PimcError
    from pimc.engine import ChainParams, Engine, Mix
    ps = [ChainParams(dim=2, N=8 + 4 * i, M=16, L=4.0, T=1.0, lam=0.5, harmonic_omega=1.0,
                      interactions=True, pair_g=1.0, pair_sigma=0.5, r_a=1.0, seed=50 + i,
                      energy_capacity=16) for i in range(3)]
    mix = Mix(stage_slices=8, stage_min=2, stage_max=8, stage_minacc=0.0, stage_maxacc=1.0,
              swaps_per_sweep=4, swap_slices=8, swap_min=2, swap_max=8, swap_minacc=0.0,
              swap_maxacc=1.0, com_phases=1, com_step=1.0, com_minstep=0.1, com_maxstep=2.0,
              adapt=1, measure_every=2)
    a = Engine(ps)
    a.set_mix(mix)
    a.run_batched(5)
    ck = str(tmp_path / "state.ckpt")
    a.save_checkpoint(ck)
    a.run_batched(7)
    b = Engine(ps)
    b.set_mix(mix)
    b.load_checkpoint(ck)
    b.run_batched(7)
    for c in range(3):
        np.testing.assert_array_equal(a.get_beads(c), b.get_beads(c))
        np.testing.assert_array_equal(a.get_next(c), b.get_next(c))
        np.testing.assert_array_equal(a.observables(c), b.observables(c))
    raw = bytearray(open(ck, "rb").read())
    raw[40] ^= 0x01
    bad = str(tmp_path / "bad.ckpt")
    open(bad, "wb").write(bytes(raw))
    with pytest.raises(PimcError, match="checksum"):
        b.load_checkpoint(bad)
    other = Engine(ps[:2])
    with pytest.raises(PimcError):
        other.load_checkpoint(ck)
    with pytest.raises(PimcError):
        b.load_checkpoint(str(tmp_path / "missing.ckpt"))
