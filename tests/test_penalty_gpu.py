"""Penalty forces on the GPU (ccd_penalty_group_force) against the golden
fixtures (made by the reference's own PenaltyGroup / PenaltyPotential) and the
oracle.

Parity bar: forces equal bit for bit (each vertex's contributions are summed
in the reference's order), identical fired flags and newused flag."""
import json
import os

import numpy as np
import pytest

import collisiondetection_gb300 as C
from collisiondetection_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from collisiondetection_gb300 import build as B

    B.build_library()
    c = C.Context(0)
    yield c
    c.close()


def _same_bits(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return (a.view(np.uint64) == b.view(np.uint64)) | (np.isnan(a) & np.isnan(b))


@pytest.mark.parametrize("scene", ["spheres", "cloth", "hand"])
def test_penalty_matches_reference(ctx, golden_dir, scene):
    meta = json.load(open(os.path.join(golden_dir, "penalty.json")))
    g = np.load(os.path.join(golden_dir, "penalty.npz"))
    p = meta[scene]
    for label, use_new in (("new", True), ("old", False)):
        F, vfire, efire, used = ctx.penalty_group_force(
            g[f"{scene}_q"], g[f"{scene}_v"], g[f"{scene}_F0"], g[f"{scene}_vf"], g[f"{scene}_ee"], p["outer_eta"],
            p["inner_eta"], p["stiffness"], p["cor"], p["dt"],
            g[f"{scene}_vf_isnew"] if use_new else None, g[f"{scene}_ee_isnew"] if use_new else None)
        bad = np.nonzero(~_same_bits(F, g[f"{scene}_{label}_F"]))[0]
        assert bad.size == 0, f"forces differ at coordinates {bad[:10]}"
        np.testing.assert_array_equal(vfire, g[f"{scene}_{label}_vf_fired"])
        np.testing.assert_array_equal(efire, g[f"{scene}_{label}_ee_fired"])
        assert used == meta[f"{scene}_{label}"]["newused"]


def test_penalty_large_group_matches_oracle(ctx, oracle):
    """A large group (sheet on sphere, 64^2 grid + level-4 sphere, every
    candidate of a wide padding) with many stencils per vertex."""
    f, frames = W.cloth_frames(grid=64, level=4, seed=8, steps=30)
    q = frames[27]
    vf, ee = oracle.broadphase(0, q, q, f, 0.03)
    rng = np.random.default_rng(4)
    vf = vf[rng.permutation(vf.shape[0])]
    ee = ee[rng.permutation(ee.shape[0])]
    v = (frames[28] - frames[26]) / 2
    F0 = rng.normal(0, 1, q.shape)
    vn = (rng.random(vf.shape[0]) < 0.01).astype(np.uint8)
    args = (q, v, F0, vf, ee, 0.03, 1e-5, 3.0, 0.3, 0.02)
    F, vfire, efire, used = ctx.penalty_group_force(*args, vf_isnew=vn)
    Fr, vfr, efr, usedr = oracle.penalty_group_force(*args, vf_isnew=vn)
    assert vfire.sum() > 100 and efire.sum() > 100
    assert _same_bits(F, Fr).all()
    np.testing.assert_array_equal(vfire, vfr)
    np.testing.assert_array_equal(efire, efr)
    assert used == usedr


def test_penalty_edge_cases(ctx, oracle):
    q = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [0.2, 0.2, 0.01]], float).ravel()
    v = np.zeros_like(q)
    F0 = np.full(q.size, -0.0)
    # no stencil: F + 0 * dt turns -0.0 into +0.0, as the reference's F += group * dt does
    F, vfire, efire, used = ctx.penalty_group_force(q, v, F0, np.zeros((0, 4)), np.zeros((0, 4)), 0.05, 0.0, 1.0,
                                                    0.5, 0.1)
    Fr = oracle.penalty_group_force(q, v, F0, np.zeros((0, 4)), np.zeros((0, 4)), 0.05, 0.0, 1.0, 0.5, 0.1)[0]
    assert _same_bits(F, Fr).all() and not used and vfire.size == 0
    with pytest.raises(C.CcdError):
        ctx.penalty_group_force(q, v, F0, [[0, 1, 2, 7]], np.zeros((0, 4)), 0.05, 0.0, 1.0, 0.5, 0.1)


def test_penalty_device_entry_point(ctx, golden_dir):
    torch = pytest.importorskip("torch")
    meta = json.load(open(os.path.join(golden_dir, "penalty.json")))
    g = np.load(os.path.join(golden_dir, "penalty.npz"))
    scene = "spheres"
    p = meta[scene]
    dev = {k: torch.from_numpy(np.ascontiguousarray(g[f"{scene}_{k}"])).cuda()
           for k in ("q", "v", "F0", "vf", "ee", "vf_isnew", "ee_isnew")}
    n_vf, n_ee = dev["vf"].shape[0], dev["ee"].shape[0]
    vfire = torch.zeros(n_vf, dtype=torch.uint8, device="cuda")
    efire = torch.zeros(n_ee, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    used = ctx.penalty_group_force_device(dev["q"].numel() // 3, dev["q"].data_ptr(), dev["v"].data_ptr(), n_vf,
                                          dev["vf"].data_ptr(), n_ee, dev["ee"].data_ptr(), p["outer_eta"],
                                          p["inner_eta"], p["stiffness"], p["cor"], p["dt"], dev["F0"].data_ptr(),
                                          vfire.data_ptr(), efire.data_ptr(), dev["vf_isnew"].data_ptr(),
                                          dev["ee_isnew"].data_ptr())
    ctx.synchronize()
    assert _same_bits(dev["F0"].cpu().numpy(), g[f"{scene}_new_F"]).all()
    np.testing.assert_array_equal(vfire.cpu().numpy(), g[f"{scene}_new_vf_fired"])
    np.testing.assert_array_equal(efire.cpu().numpy(), g[f"{scene}_new_ee_fired"])
    assert used == meta[f"{scene}_new"]["newused"]
    # an index out of range is caught by the kernel's own check, F stays as it was
    before = dev["F0"].clone()
    bad = dev["vf"][:4].clone()
    bad[2, 3] = dev["q"].numel() // 3 + 5
    with pytest.raises(C.CcdError):
        ctx.penalty_group_force_device(dev["q"].numel() // 3, dev["q"].data_ptr(), dev["v"].data_ptr(), 4,
                                       bad.data_ptr(), 0, dev["ee"].data_ptr(), p["outer_eta"], p["inner_eta"],
                                       p["stiffness"], p["cor"], p["dt"], dev["F0"].data_ptr(), vfire.data_ptr(),
                                       efire.data_ptr())
    ctx.synchronize()
    assert torch.equal(before, dev["F0"])
