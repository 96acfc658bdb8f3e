"""The random numbers of the device-resident Metropolis run, restated on the CPU and pinned to the
reference's recorded argon run.

The device run (k_replay, mc_cpp_gb300/csrc/single.cu) turns the host generator's raw std::mt19937
words into doubles as libstdc++'s generate_canonical<double, 53> does: two words, w0 + w1 2^32
rounded once, times 2^-64, a result of 1 replaced by the largest double below 1.  Its draw order is
MC_metropolis::run's (MC.cpp:142-156, MC_metropolis.cpp:175-204): the move type, the instance, unit
ball tries of three uniforms (2u - 1 each) until one lies in the ball, the displacement scaled by
dmax, and a uniform for the acceptance test only when dE > DBL_EPSILON.  numpy's MT19937 with the
legacy seeding produces std::mt19937's words.  Checked on all 2,000 steps of the reference's argon
trace (tests/golden/trace_argon864.npy): the moved atom, the displacement and the acceptance
uniform, bit for bit.
"""
import numpy as np
import pytest

import goldens

DBL_EPS = 2.220446049250313e-16


def _words(seed):
    g = np.random.MT19937()
    g._legacy_seeding(seed)
    while True:
        yield int(g.random_raw())


def _canonical(it):
    """generate_canonical<double, 53> on two words, as the device forms it."""
    w0, w1 = next(it), next(it)
    r = (float(w0) + float(w1) * 4294967296.0) * 5.421010862427522170037264e-20
    return r if r < 1.0 else float(np.nextafter(1.0, 0.0))


def test_mt19937_words_are_the_standard_ones():
    it = _words(5489)                                  # std::mt19937's default seed
    first = [next(it) for _ in range(10000)]
    assert first[0] == 3499211612
    assert first[9999] == 4123659995                   # the value the C++ standard requires


def test_device_draws_reproduce_the_reference_argon_trace():
    g = goldens.golden()["mc"]["argon864"]
    s = goldens.system("argon864")
    (mv,) = s.moves
    assert mv.move_type == "trn" and mv.dmax_each == 0
    ninst, dmax = s.natom, float(mv.dmax_value)
    tr = goldens.trace("argon864")
    it = _words(int(g["seed"]))
    for k in range(len(tr)):
        typ = int(1.0 * _canonical(it))
        inst = int(float(ninst) * _canonical(it))
        while True:
            rx = _canonical(it) * 2.0 - 1.0
            ry = _canonical(it) * 2.0 - 1.0
            rz = _canonical(it) * 2.0 - 1.0
            if (rx * rx + ry * ry) + rz * rz <= 1.0:
                break
        row = tr[k]
        assert (typ, inst) == (int(row[1]), int(row[2])), k
        assert (rx * dmax, ry * dmax, rz * dmax) == (row[3], row[4], row[5]), k
        alpha = _canonical(it) if row[9] > DBL_EPS else -1.0
        assert alpha == row[10], (k, alpha, row[10])
