"""The oracle restatement against the reference's own sources compiled here
(oracle/_ref, built by oracle/Makefile from the reference tree), directly on
seeded workloads larger than the committed fixtures.  CPU only; skipped
where the reference build is absent (it does not travel with the tests).

Bar: identical hit flags and candidate sets; contact times bit-identical
(both sides use the host's exp/log)."""
import numpy as np
import pytest

from collisiondetection_gb300 import workloads as W

import oracle as O

pytestmark = pytest.mark.skipif(not O.Reference.available(), reason="the reference build (oracle/_ref) is absent")


@pytest.fixture(scope="module")
def ref():
    return O.Reference()


@pytest.mark.parametrize("kind", [W.KIND_VF, W.KIND_EE, W.KIND_VE, W.KIND_VV])
def test_primitive_batches_bit_identical(oracle, ref, kind):
    n = 60_000
    x = W.primitive_batch(kind, n, seed=500 + kind)
    eta = 10.0 ** np.random.default_rng(kind).uniform(-8, -3, n)
    for e in (1e-6, eta):
        h_o, t_o = oracle.batch(kind, x, e, nthreads=4)
        h_r, t_r = ref.batch(kind, x, e)
        assert np.array_equal(h_o, h_r)
        m = h_r == 1
        assert m.sum() > 100
        assert np.array_equal(t_o[m].view(np.uint64), t_r[m].view(np.uint64))


def test_cloth_frame_broad_and_narrow_phase(oracle, ref):
    q0, q1, faces = W.sheet_on_sphere(grid=24, level=3, seed=3, step=2, gap=0.004, drop=0.004, wrinkle=0.003)
    for kind in (0, 1):  # k-DOP, AABB
        vf_o, ee_o = oracle.broadphase(kind, q0, q1, faces, 1e-3)
        vf_r, ee_r = ref.broadphase(kind, q0, q1, faces, 1e-3)
        assert np.array_equal(vf_o, vf_r) and np.array_equal(ee_o, ee_r)
        assert vf_r.shape[0] > 0 and ee_r.shape[0] > 0
    out = oracle.narrowphase(q0, q1, vf_r, 1e-3, ee_r, 1e-3)
    vh, eh = ref.narrowphase(q0, q1, vf_r, 1e-3, ee_r, 1e-3)
    assert np.array_equal(out["vf_hit"], vh) and np.array_equal(out["ee_hit"], eh)
    assert vh.sum() > 0 and eh.sum() > 0


def test_uneven_instances_broad_phase(oracle, ref):
    faces, frames, _, _ = W.uneven_batch(n_instances=4, lo=200, hi=1500, seed=9, steps=1)
    vf_o, ee_o = oracle.broadphase(0, frames[0], frames[1], faces, 1e-6)
    vf_r, ee_r = ref.broadphase(0, frames[0], frames[1], faces, 1e-6)
    assert np.array_equal(vf_o, vf_r) and np.array_equal(ee_o, ee_r)
