"""Differentiable density calibration on the GPU: the hand-written adjoint against
the FP64 CPU adjoint about the same FP32 trajectory, central finite differences
(step 1e-3) of the GPU forward, determinism and the autograd path.

The FP32 forward is a staircase at the 1e-3 scale: a speed change of 1e-3 moves a
tick's step by 1e-4 m while positions of a few hundred metres have an ulp of
3e-5..6e-5 m, so single central differences of the FP32 loss carry a few per cent
of rounding noise.  The finite-difference checks here are therefore statistical
(correlation, slope, norm-wise error over 64 parameters); the tight check of the
adjoint's arithmetic is the FP64 comparison (1e-4 relative), and the FP64 adjoint
itself is pinned to central differences of the smooth FP64 model in
tests/test_oracle.py."""
import importlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REL_TOL_F64 = 1e-4  # gradients within 1e-4 relative (norm-wise) of the FP64 reference
H = 1e-3            # finite-difference step


def _setup(msim, torch, n=6000, ticks=300, side=16, grid=(64, 64), K=50, seed=5, rng="pcg32"):
    cal_mod = importlib.import_module("movement-sim_gb300.calibration")
    road_map = msim.RoadMap.lattice(side, seed)
    calib = cal_mod.Calibration(road_map, n, ticks, dt=0.1, rng=rng, checkpoint_interval=K, grid=grid,
                                seed=seed, placement="fraction", speed=(1.0, 1.6))
    rs = np.random.default_rng(seed)
    hidden = rs.uniform(0.7, 1.3, road_map.num_roads).astype(np.float32)
    G = grid[0] * grid[1]
    target = torch.empty(G, dtype=torch.float32, device="cuda")
    calib.forward(factor=torch.from_numpy(hidden).cuda(), density=target)  # target from hidden factors
    st = calib.initial_state()
    speed = torch.from_numpy(st["speed"].copy()).cuda()
    factor = torch.ones(road_map.num_roads, dtype=torch.float32, device="cuda")
    return cal_mod, road_map, calib, st, speed, factor, target


@pytest.mark.parametrize("rng,rng_kind,K", [("pcg32", 1, 50), ("xorshift128", 0, 64)])
def test_adjoint_matches_fp64_reference(msim, orc, rng, rng_kind, K):
    torch = pytest.importorskip("torch")
    cal_mod, road_map, calib, st, speed, factor, target = _setup(msim, torch, rng=rng, K=K)
    with calib:
        loss = calib.forward(speed, factor, target)
        gs = torch.empty(calib.n, dtype=torch.float32, device="cuda")
        gf = torch.empty(road_map.num_roads, dtype=torch.float32, device="cuda")
        calib.backward(gs, gf)
        gs64, gf64 = calib.gradients_f64()
        # determinism: a second backward is bit-identical
        gs2 = torch.empty_like(gs)
        gf2 = torch.empty_like(gf)
        calib.backward(gs2, gf2)
        assert torch.equal(gs, gs2) and torch.equal(gf, gf2)
        dens = torch.empty(calib.grid[0] * calib.grid[1], dtype=torch.float32, device="cuda")
        loss2 = calib.forward(speed, factor, target, density=dens)
        assert loss2 == loss
    rl, rdens, rgs, rgf = orc.density_adjoint(road_map, st, speed.cpu().numpy(), factor.cpu().numpy(), rng_kind, 0.1,
                                              calib.ticks, calib.grid, target.cpu().numpy())
    assert abs(loss - rl) <= 1e-6 * abs(rl)
    np.testing.assert_allclose(dens.cpu().numpy(), rdens, rtol=1e-5, atol=1e-7 * rdens.max())
    for g, r in ((gs64, rgs), (gf64, rgf)):
        err = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert err < REL_TOL_F64, err
        assert np.abs(g - r).max() <= 1e-3 * np.abs(r).max()
    assert np.abs(gf64).max() > 0 and np.abs(gs64).max() > 0
    np.testing.assert_array_equal(gs.cpu().numpy(), gs64.astype(np.float32))
    np.testing.assert_array_equal(gf.cpu().numpy(), gf64.astype(np.float32))


def _fd_stats(fd, g):
    fd, g = np.asarray(fd), np.asarray(g)
    return (float(np.corrcoef(fd, g)[0, 1]), float(np.linalg.norm(fd - g) / np.linalg.norm(g)),
            float(fd @ g / (g @ g)))


def test_finite_differences(msim):
    """Central differences (step 1e-3) of the GPU forward on 64 random parameters:
    32 speeds and 32 road factors whose +-1e-3 natural runs cross no road-end event
    (the recorded event schedule is unchanged); and on parameters drawn without that
    selection, with the forward's events replayed."""
    torch = pytest.importorskip("torch")
    cal_mod, road_map, calib, st, speed, factor, target = _setup(msim, torch, n=3000, ticks=200)
    rs = np.random.default_rng(11)
    with calib:
        calib.forward(speed, factor, target, mode="record")
        base = calib.schedule()
        gs = torch.empty(calib.n, dtype=torch.float32, device="cuda")
        gf = torch.empty(road_map.num_roads, dtype=torch.float32, device="cuda")
        calib.backward(gs, gf)
        grads = dict(zip(("speed", "factor"), calib.gradients_f64()))
        vecs = {"speed": speed, "factor": factor}
        for kind in ("speed", "factor"):
            vec, grad = vecs[kind], grads[kind]
            fds, gg = [], []
            for i in rs.permutation(vec.numel())[:400]:
                v0 = float(vec[i])
                res, used = [], []
                for d in (H, -H):
                    vec[i] = v0 + d
                    used.append(float(vec[i]))  # the float32 value actually used
                    res.append(calib.forward(speed, factor, target, mode="record"))
                    if not np.array_equal(calib.schedule(), base):
                        break
                vec[i] = v0
                if len(res) < 2 or not np.array_equal(calib.schedule(), base):
                    continue
                fds.append((res[0] - res[1]) / (used[0] - used[1]))
                gg.append(grad[i])
                if len(fds) == 32:
                    break
            assert len(fds) == 32, (kind, len(fds))
            corr, l2, slope = _fd_stats(fds, gg)
            assert corr > 0.99 and l2 < 0.15 and 0.9 < slope < 1.1, (kind, corr, l2, slope)
        # replayed events: no selection needed
        calib.forward(speed, factor, target, mode="record")
        for kind in ("speed", "factor"):
            vec, grad = vecs[kind], grads[kind]
            fds, gg = [], []
            for i in rs.choice(vec.numel(), 16, replace=False):
                v0 = float(vec[i])
                vec[i] = v0 + H
                vp = float(vec[i])
                lp = calib.forward(speed, factor, target, mode="replay")
                vec[i] = v0 - H
                vm = float(vec[i])
                lm = calib.forward(speed, factor, target, mode="replay")
                vec[i] = v0
                fds.append((lp - lm) / (vp - vm))
                gg.append(grad[i])
            corr, l2, slope = _fd_stats(fds, gg)
            assert corr > 0.98 and l2 < 0.2 and 0.85 < slope < 1.15, (kind, corr, l2, slope)


def test_autograd_function(msim):
    torch = pytest.importorskip("torch")
    cal_mod, road_map, calib, st, speed, factor, target = _setup(msim, torch, n=3000, ticks=150)
    with calib:
        s = speed.clone().requires_grad_(True)
        f = factor.clone().requires_grad_(True)
        loss = cal_mod.density_loss(calib, s, f, target)
        loss.backward()
        gs = torch.empty(calib.n, dtype=torch.float32, device="cuda")
        gf = torch.empty(road_map.num_roads, dtype=torch.float32, device="cuda")
        calib.forward(speed, factor, target)
        calib.backward(gs, gf)
        assert torch.equal(s.grad, gs) and torch.equal(f.grad, gf)
        # one descent step on the factors lowers the loss
        with torch.no_grad():
            f2 = f - 0.5 * f.grad / f.grad.abs().max()
        assert calib.forward(speed, f2.contiguous(), target) < float(loss)


def test_adjoint_rejects_bad_arguments(msim):
    torch = pytest.importorskip("torch")
    cal_mod = importlib.import_module("movement-sim_gb300.calibration")
    road_map = msim.RoadMap.lattice(8, 1)
    with pytest.raises(Exception):
        cal_mod.Calibration(road_map, 0, 10)
    with pytest.raises(Exception):
        cal_mod.Calibration(road_map, 100, 0)
    with cal_mod.Calibration(road_map, 100, 20, checkpoint_interval=7, grid=(8, 8)) as calib:
        with pytest.raises(Exception):
            calib.backward()  # no forward yet
        with pytest.raises(Exception):
            calib.forward(mode="replay")  # nothing recorded
        with pytest.raises(ValueError):
            calib.forward(speed=torch.ones(99, device="cuda"))
        assert calib.forward() >= 0.0
