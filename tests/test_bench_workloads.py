"""The benchmark's workloads against the sizes of the configurations they
stand for (node, equation and element counts, multigrid levels), and the
seeded initial temperatures (reproducible, boundary values in place)."""
import numpy as np

import bench


def test_headline_64_cubed():
    c = bench.workload(64)
    assert (c.nox, c.noy, c.noz, c.levels) == (65, 65, 65, 5)
    assert c.nno == 274625 and 3 * c.nno == 823875
    assert bench.bytes_per_sweep(c.nno, 4) == 274625 * 4 * 276


def test_cfg2_box():
    c = bench.cfg2_workload()
    assert (c.nox, c.noy, c.noz, c.levels) == (129, 129, 65, 6)
    assert c.nno == 1081665 and c.dimen == (2.0, 2.0, 1.0) and c.Q0 == 1.0
    assert c.visc0 == (1.0, 30.0) and c.z_layer == (0.8,)


def test_sphere_segment():
    c = bench.sphere_workload()
    assert (c.nox, c.noy, c.noz, c.levels) == (193, 193, 97, 6)
    assert c.nno == 3613153


def test_seeded_T0():
    c = bench.workload(64)
    a, b = bench.seeded_T0(c, 0), bench.seeded_T0(c, 0)
    assert np.array_equal(a, b) and not np.array_equal(a, bench.seeded_T0(c, 1))
    T = a.reshape(c.noy, c.nox, c.noz)
    assert np.all(T[:, :, 0] == 1.0) and np.all(T[:, :, -1] == 0.0)
    assert np.max(np.abs(T[:, :, 1:-1] - (1.0 - np.linspace(0, 1, c.noz)[1:-1]))) <= 0.01
    s = bench.sphere_workload()
    Ts = bench.seeded_T0_sphere(s, 0).reshape(s.noy, s.nox, s.noz)
    assert np.all(Ts[:, :, 0] == 1.0) and np.all(Ts[:, :, -1] == 0.0)
