"""Learned warm start on the GPU: input assembly, forward, loss, the full
backward (every parameter gradient) and Adam against the torch-CPU oracle
(oracle/unet_oracle.py), the fluid-cell norm option, and training."""
import numpy as np
import pytest

from oracle import unet_oracle as U

pytestmark = pytest.mark.gpu


def _planes_from_solver(imax=32, jmax=32, steps=3, batch=2):
    """Real solver planes: a small channel with one obstacle, `batch`
    consecutive steps exported between tick_prepare and tick_solve."""
    from stroemung_gb300 import presets, warmstart
    grid = presets.channel(imax, jmax, [(12, 12, 6, 5)])
    sim = warmstart.make_simulation(grid, 200.0, 0.01, max_iterations=200)
    planes = warmstart.PlaneBatch(batch, imax + 2, jmax + 2)
    for _ in range(steps - batch):
        sim.run_simulation_tick()
    for i in range(batch):
        sim.tick_prepare()
        warmstart.export_sample(sim, planes, i)
        sim.tick_solve()
    sim.close()
    return planes


def _net_with_random_head(seed=3):
    import torch
    from stroemung_gb300.unet import UNet
    net = UNet(seed=seed)
    th = net.theta.detach().cpu().numpy().copy()
    rng = np.random.default_rng(seed)
    th[-33:] = rng.normal(0.0, 0.3, 33).astype(np.float32)
    net.load_state_dict({"theta": th, "step": 0})
    torch.cuda.synchronize()
    return net, th


def test_unet_parameter_layout_matches_oracle():
    from stroemung_gb300.unet import UNet
    net = UNet(seed=0)
    expected = sum((-(-9 * (-(-ci // 8) * 8) // 64) * 64) * co + co
                   for ci, co in U.conv_shapes()) + 33
    assert net.n_params == expected
    convs, wh, bh = U.unpack(net.theta.detach().cpu().numpy())
    assert len(convs) == 14 and wh.numel() == 32 and bh.numel() == 1
    # the head starts at zero, the convolutions He-initialised
    assert float(wh.abs().max()) == 0.0 and float(convs[0][0].abs().max()) > 0.0


def test_prepare_input_matches_oracle():
    import torch
    from stroemung_gb300 import warmstart
    from stroemung_gb300.unet import UNet
    planes = _planes_from_solver()
    net = UNet(seed=0)
    tr = warmstart.Trainer(net, planes.nx, planes.ny, 0.01, 0.01, batch=2)
    rhs, flags, pprev = (planes.rhs.cpu().numpy(), planes.flags.cpu().numpy(),
                         planes.p.cpu().numpy())
    tr.loss(planes, 0)
    torch.cuda.synchronize()
    xin_ref, s_ref, mean_ref = U.prepare_input(rhs, flags, pprev, 1e-4)
    np.testing.assert_allclose(tr.smax.cpu().numpy(), s_ref.numpy(), rtol=1e-6)
    np.testing.assert_allclose(tr.pmean.cpu().numpy(), mean_ref.numpy(), rtol=1e-4, atol=1e-6)
    got = tr.xin.float().cpu().numpy()
    ref = xin_ref.numpy()
    # one BF16 ulp where the FP32 mean differs in its last bits
    np.testing.assert_allclose(got, ref, rtol=1e-2, atol=1e-3)
    assert np.mean(got == ref) > 0.98


def test_forward_loss_and_every_gradient_match_oracle():
    """GPU forward + relative-residual loss + backward (tcgen05 wgrad and
    dgrad, pooling / upsampling adjoints, head, loss adjoint) vs torch
    autograd on the same BF16-rounded network.  Tolerances: q and the loss
    within 2e-2 relative (BF16 activations, different summation order),
    every layer's weight and bias gradient within twice that layer's own BF16
    noise (the oracle's BF16-rounded gradient against its plain FP32 one;
    both sides round activation gradients to BF16 where the kernels store
    them, summation orders differ) plus 1e-2, relative L2, and cosine > 0.99."""
    import torch
    from stroemung_gb300 import warmstart
    planes = _planes_from_solver()
    net, theta = _net_with_random_head()
    tr = warmstart.Trainer(net, planes.nx, planes.ny, 0.01, 0.01, batch=2)
    rhs, flags, pprev = (planes.rhs.cpu().numpy(), planes.flags.cpu().numpy(),
                         planes.p.cpu().numpy())
    loss_gpu, per_gpu = tr.loss(planes, 0)
    q_gpu = net._bufs[(2, planes.nx - 2, planes.ny - 2)]["q"].cpu().numpy()
    net.zero_grad()
    L = net.L
    net._check(L.strm_nn_residual_loss_grad(tr.r.data_ptr(), planes.flags.data_ptr(),
                                            tr.sum_b2.data_ptr(), tr.smax.data_ptr(), tr.dx2,
                                            tr.rdx2, tr.rdy2, tr.gp.data_ptr(), tr.gq.data_ptr(),
                                            2, planes.nx, planes.ny, None), "loss grad")
    net.backward(tr.gq, 2, planes.nx - 2, planes.ny - 2)
    torch.cuda.synchronize()
    g_gpu = net.grad.cpu().numpy()

    loss_ref, per_ref, q_ref, g_ref = U.loss_and_grads(theta, rhs, flags, pprev, 0.01, 0.01)
    _, _, _, g_fp32 = U.loss_and_grads(theta, rhs, flags, pprev, 0.01, 0.01, bf16=False)
    assert np.linalg.norm(q_gpu - q_ref) <= 2e-2 * np.linalg.norm(q_ref)
    np.testing.assert_allclose(per_gpu, per_ref, rtol=2e-2)
    assert abs(loss_gpu - loss_ref) <= 2e-2 * loss_ref
    names = [f"conv{i}.{k}" for i in range(14) for k in ("w", "b")] + ["head.w", "head.b"]
    sizes = []
    for ci, co in U.conv_shapes():
        kp = -(-9 * (-(-ci // 8) * 8) // 64) * 64
        sizes += [co * kp, co]
    sizes += [32, 1]
    assert sum(sizes) == g_gpu.size
    stats, bad = [], []
    o = 0
    for name, n in zip(names, sizes):
        a, b, c = (g[o:o + n].astype(np.float64) for g in (g_gpu, g_ref, g_fp32))
        o += n
        if name == "head.b":
            # a constant added to q on every fluid cell leaves the residual
            # unchanged (pure Neumann problem): this gradient is 0 up to rounding
            scale = np.linalg.norm(g_gpu[o - 33:o - 1])
            if not (abs(a[0]) <= 1e-2 * scale and abs(b[0]) <= 1e-2 * scale):
                bad.append((name, a[0], b[0], scale))
            continue
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        noise = np.linalg.norm(b - c) / np.linalg.norm(c)  # the layer's own BF16 noise
        stats.append((name, round(rel, 4), round(cos, 5), round(noise, 4)))
        if not (rel <= 2.0 * noise + 1e-2 and cos >= 0.99):
            bad.append(stats[-1])
    print("per-layer gradient (name, rel L2 vs oracle, cosine, BF16 noise):", stats)
    assert not bad, bad


def test_adam_matches_oracle():
    import torch
    from stroemung_gb300 import _lib
    L = _lib.load()
    rng = np.random.default_rng(5)
    n = 10007
    th = rng.normal(size=n).astype(np.float32)
    gr = rng.normal(size=n).astype(np.float32)
    m = rng.normal(size=n).astype(np.float32) * 0.1
    v = np.abs(rng.normal(size=n)).astype(np.float32) * 0.01
    t = [torch.tensor(a, device="cuda") for a in (th, gr, m, v)]
    wbf = torch.empty(n, dtype=torch.bfloat16, device="cuda")
    assert L.strm_nn_adam(t[0].data_ptr(), t[1].data_ptr(), t[2].data_ptr(), t[3].data_ptr(), n,
                          1e-3, 0.9, 0.999, 1e-8, 7, wbf.data_ptr(), None) == 0
    torch.cuda.synchronize()
    th2, m2, v2 = U.adam(th, gr, m, v, 7, 1e-3)
    np.testing.assert_allclose(t[2].cpu().numpy(), m2, rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(t[3].cpu().numpy(), v2, rtol=1e-6, atol=1e-9)
    np.testing.assert_allclose(t[0].cpu().numpy(), th2, rtol=1e-6, atol=1e-6)
    np.testing.assert_array_equal(wbf.float().cpu().numpy(),
                                  t[0].to(torch.bfloat16).float().cpu().numpy())


def test_fluid_norm_excludes_obstacles():
    """The fluid-cell norm equals the residual sum over fluid cells only; the
    reference norm includes obstacle cells."""
    from stroemung_gb300 import presets
    from stroemung_gb300.simulation import (NORM_ALL_INTERIOR, NORM_FLUID, NORM_FLUID_MEAN_FREE,
                                            Simulation)
    grid = presets.channel(48, 24, [(20, 8, 6, 6)])
    sim = Simulation(grid=grid, cell_size=(0.01, 0.01), delt=0.005, gamma=0.9, reynolds=100.0,
                     max_iterations=50, tau=0.5)
    for _ in range(3):
        sim.run_simulation_tick()
    sim.copy_pressure_to_boundaries()
    p, rhs = sim.download("p"), sim.download("rhs")
    dx2 = 0.01 * 0.01
    r = ((p[2:, 1:-1] - p[1:-1, 1:-1]) - (p[1:-1, 1:-1] - p[:-2, 1:-1])) / dx2 + \
        ((p[1:-1, 2:] - p[1:-1, 1:-1]) - (p[1:-1, 1:-1] - p[1:-1, :-2])) / dx2 - rhs[1:-1, 1:-1]
    fluid = sim._kind[1:-1, 1:-1] == 0
    nf = float(sim.state()["fluid_cells"])
    ns_all = sim.calculate_norm_squared()
    sim.set_mode(norm_cells=NORM_FLUID, strict_eps=True)
    ns_fluid = sim.calculate_norm_squared()
    sim.set_mode(norm_cells=NORM_FLUID_MEAN_FREE, strict_eps=True)
    ns_mf = sim.calculate_norm_squared()
    np.testing.assert_allclose(ns_all, (r ** 2).sum() / nf, rtol=1e-10)
    np.testing.assert_allclose(ns_fluid, (r[fluid] ** 2).sum() / nf, rtol=1e-10)
    rf = r[fluid]
    np.testing.assert_allclose(ns_mf, ((rf ** 2).sum() - rf.sum() ** 2 / nf) / nf, rtol=1e-9)
    assert ns_mf <= ns_fluid < ns_all
    # the residual's fluid sum is -sum(rhs): the Laplacian with the boundary
    # copy sums to zero over fluid cells
    np.testing.assert_allclose(rf.sum(), -rhs[1:-1, 1:-1][fluid].sum(),
                               rtol=1e-6, atol=1e-6 * np.abs(rf).sum())
    sim.set_mode(norm_cells=NORM_ALL_INTERIOR)
    sim.close()


def test_training_lowers_the_loss():
    """A few hundred Adam steps on solver snapshots lower the relative
    residual of the corrected pressure on held-out snapshots."""
    from stroemung_gb300 import warmstart
    from stroemung_gb300.unet import UNet
    train = warmstart.generate_snapshots(256, imax=64, jmax=32, steps_per_problem=16, seed=1,
                                         max_iterations=300)
    held = warmstart.generate_snapshots(32, imax=64, jmax=32, steps_per_problem=16, seed=2,
                                        max_iterations=300)
    net = UNet(seed=0)
    tr = warmstart.Trainer(net, 66, 34, 0.01, 0.01, batch=32)
    before, _ = tr.loss(held, 0)
    tr.fit(train, epochs=40, lr=1e-3)
    after, _ = tr.loss(held, 0)
    assert after < 0.8 * before, (before, after)


def test_error_loss_and_gradient_match_numpy():
    """strm_nn_error_loss: relative mean-free error of the corrected pressure
    against a target on fluid interior cells, and its gradient with respect
    to q, against a float64 numpy restatement."""
    import torch
    from stroemung_gb300 import _lib
    L = _lib.load()
    b, nx, ny, dx2 = 3, 20, 14, 1e-4
    rng = np.random.default_rng(7)
    pprev = rng.normal(size=(b, nx, ny)).astype(np.float32)
    pt = (pprev + 0.1 * rng.normal(size=(b, nx, ny))).astype(np.float32)
    q = rng.normal(size=(b, nx - 2, ny - 2)).astype(np.float32)
    flags = np.zeros((b, nx, ny), np.uint8)
    flags[:, 0, :] = flags[:, -1, :] = flags[:, :, 0] = flags[:, :, -1] = 1
    flags[:, 6:9, 4:7] = 1 | (2 << 3)
    smax = np.array([50.0, 0.0, 3.0], np.float32)  # a zero scale counts as 1
    dev = lambda a: torch.from_numpy(a).cuda()  # noqa: E731
    t_pp, t_pt, t_q, t_fl, t_s = dev(pprev), dev(pt), dev(q), dev(flags), dev(smax)
    work = torch.zeros(5 * b, dtype=torch.float32, device="cuda")
    loss = torch.zeros(b, dtype=torch.float32, device="cuda")
    gq = torch.zeros_like(t_q)
    assert L.strm_nn_error_loss(t_pp.data_ptr(), t_q.data_ptr(), t_pt.data_ptr(), t_fl.data_ptr(),
                                t_s.data_ptr(), dx2, work.data_ptr(), loss.data_ptr(),
                                gq.data_ptr(), b, nx, ny, None) == 0
    torch.cuda.synchronize()
    s = np.where(smax > 0, smax, 1.0).astype(np.float64)
    fl = flags[:, 1:-1, 1:-1] == 0
    want_loss = np.zeros(b)
    want_g = np.zeros((b, nx - 2, ny - 2))
    for k in range(b):
        e = pprev[k, 1:-1, 1:-1] + s[k] * dx2 * q[k] - pt[k, 1:-1, 1:-1]
        d = pt[k, 1:-1, 1:-1] - pprev[k, 1:-1, 1:-1]
        em = e[fl[k]] - e[fl[k]].mean()
        dm = d[fl[k]] - d[fl[k]].mean()
        want_loss[k] = (em ** 2).sum() / (dm ** 2).sum()
        want_g[k][fl[k]] = 2.0 / b * em / (dm ** 2).sum() * s[k] * dx2
    np.testing.assert_allclose(loss.cpu().numpy(), want_loss, rtol=1e-4)
    np.testing.assert_allclose(gq.cpu().numpy(), want_g, rtol=1e-3,
                               atol=1e-4 * np.abs(want_g).max())
    # the gradient is the derivative of the batch-mean loss: a finite
    # difference along it agrees
    h = 0.1
    qs = (q + h * want_g / np.abs(want_g).max()).astype(np.float32)
    t_q.copy_(dev(qs))
    assert L.strm_nn_error_loss(t_pp.data_ptr(), t_q.data_ptr(), t_pt.data_ptr(), t_fl.data_ptr(),
                                t_s.data_ptr(), dx2, work.data_ptr(), loss.data_ptr(), None,
                                b, nx, ny, None) == 0
    torch.cuda.synchronize()
    dl = loss.cpu().numpy().mean() - want_loss.mean()
    pred = h * (want_g ** 2).sum() / np.abs(want_g).max()
    assert abs(dl - pred) <= 0.05 * abs(pred), (dl, pred)


def test_learned_warm_start_saves_sweeps_on_cavities():
    """Trained on solved pressures of 64 x 64 lid-driven cavities (error
    loss) and judged after 16 red-black iterations, the network's correction
    brings a held-out cavity to the strict stop rule in fewer sweeps than the
    plain solve from the previous pressure, stepped A/B from identical
    states; the fields stay those of the plain run."""
    import torch
    from stroemung_gb300 import presets, warmstart
    from stroemung_gb300.unet import UNet
    n = 64
    fam = warmstart.cavity_family(n)
    train = warmstart.generate_snapshots(512, family=fam, steps_per_problem=32, seed=1,
                                         targets=True)
    net = UNet(seed=0)
    tr = warmstart.Trainer(net, n + 2, n + 2, 1.0 / n, 1.0 / n, batch=32, loss="error")
    tr.fit(train, epochs=25, lr=1e-3)
    cfg = dict(delt=1e-3, max_iterations=40000)
    plain = warmstart.make_simulation(presets.cavity(n), 400.0, 1.0 / n, **cfg)
    wsim = warmstart.make_simulation(presets.cavity(n), 400.0, 1.0 / n, **cfg)
    ws = warmstart.WarmStartSolver(wsim, net, judge_sweeps=16)
    scratch = torch.zeros(n + 2, n + 2, dtype=torch.float64, device="cuda")
    sp = sw = 0
    for _ in range(16):
        r = warmstart.compare_step(plain, ws, scratch)
        assert r["ns_plain"] < 1e-6 and r["ns_ws"] < 1e-6
        sp += r["sweeps_plain"]
        sw += r["sweeps_ws"]
    plain.close()
    wsim.close()
    assert sw <= 0.95 * sp, (sp, sw)


def test_recorded_forward_equals_forward():
    """forward_graphed replays the forward from a CUDA graph: the same bits
    as forward(keep=False), on the first call, on replays, and after the
    forward pool grew (the recording is made again)."""
    import torch
    net, _ = _net_with_random_head(seed=4)
    g = torch.Generator(device="cuda").manual_seed(6)
    x = torch.randn(1, 64, 48, 8, device="cuda", generator=g).to(torch.bfloat16)
    big = torch.randn(1, 128, 96, 8, device="cuda", generator=g).to(torch.bfloat16)
    want = net.forward(x, 1, 64, 48, keep=False).clone()
    for _ in range(3):
        got = net.forward_graphed(x, 1, 64, 48).clone()
        assert torch.equal(got, want)
    net.forward(big, 1, 128, 96, keep=False)
    x.mul_(-1.0)  # the recording reads the input buffer at replay time
    want = net.forward(x, 1, 64, 48, keep=False).clone()
    assert torch.equal(net.forward_graphed(x, 1, 64, 48).clone(), want)


def test_prediction_forward_equals_training_forward_on_tma_layers():
    """At a size whose full-resolution layers take the TMA-fed convolutions
    (rows of whole 128-pixel tiles), the prediction's forward (no
    activations kept; the last layer's outputs not stored, the head fused
    into its epilogue) gives the bits of the training forward, which stores
    every activation, and its recorded graph the same again."""
    import torch
    net, _ = _net_with_random_head(seed=5)
    g = torch.Generator(device="cuda").manual_seed(8)
    x = torch.randn(2, 64, 256, 8, device="cuda", generator=g).to(torch.bfloat16)
    keep = net.forward(x, 2, 64, 256, keep=True).clone()
    pred = net.forward(x, 2, 64, 256, keep=False).clone()
    assert torch.isfinite(keep).all()
    assert torch.equal(pred, keep)
    x1 = x[:1].contiguous()
    want = net.forward(x1, 1, 64, 256, keep=True).clone()
    assert torch.equal(net.forward_graphed(x1, 1, 64, 256).clone(), want)
    assert torch.equal(want, keep[:1])


@pytest.mark.parametrize("sweeps", [0, 4])
def test_judge_matches_the_phase_entry_points(sweeps):
    """strm_judge_correction, its launches recorded as one CUDA graph, gives
    the norms the phase entry points give for the two candidates (the
    previous pressure and the corrected one, each after the boundary copy
    and `sweeps` FP64 red-black iterations), leaves the pressure at the
    better candidate without the judge's sweeps, and does the same on a
    second call (a replay)."""
    import ctypes
    import torch
    from stroemung_gb300 import _lib, presets
    from stroemung_gb300.simulation import ARITH_FAST, Simulation
    grid = presets.channel(96, 40, [(30, 12, 8, 6), (60, 20, 5, 9)])
    sim = Simulation(grid=grid, cell_size=(0.01, 0.01), delt=0.002, gamma=0.9, reynolds=200.0,
                     max_iterations=50, tau=0.5, arithmetic=ARITH_FAST)
    sim.run_simulation_tick()
    sim.tick_prepare()
    nx, ny = sim.size
    p0 = sim.download("p")
    g = torch.Generator(device="cuda").manual_seed(3)
    q = torch.randn(nx - 2, ny - 2, device="cuda", generator=g, dtype=torch.float32)
    fluid = grid["kind"][1:-1, 1:-1] == 0
    qn = q.cpu().numpy().astype(np.float64)

    def candidate(scale):
        p = p0.copy()
        p[1:-1, 1:-1] = np.where(fluid, p[1:-1, 1:-1] + scale * qn, p[1:-1, 1:-1])
        return p

    def norm_and_field(p):
        sim.upload("p", p)
        sim.copy_pressure_to_boundaries()
        field = sim.download("p")
        ns = sim.sor_sweeps(sweeps) if sweeps else sim.calculate_norm_squared()
        return ns, field

    L = _lib.load()
    for scale in (1e-4, -3e-2):
        nb, fb = norm_and_field(candidate(scale))
        na, fa = norm_and_field(p0)
        for _ in range(2):
            sim.upload("p", p0)
            a, b, acc = ctypes.c_double(), ctypes.c_double(), ctypes.c_int()
            _lib.check(L.strm_judge_correction(sim._h, q.data_ptr(), scale, sweeps,
                                               ctypes.byref(a), ctypes.byref(b),
                                               ctypes.byref(acc)))
            assert (a.value, b.value) == (na, nb)
            assert acc.value == (1 if nb < na else 0)
            want = fb if nb < na else fa
            assert np.array_equal(sim.download("p").view(np.int64), want.view(np.int64))
    sim.close()
