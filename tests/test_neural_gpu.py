"""The learned collision proxy on the GPU: the tensor-core forward pass against a NumPy forward pass,
training on the method's own grid SDFs, and collision through the proxy against grid collision."""
import math

import numpy as np
import pytest

import nsdf_ref as R

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [1, 0], ids=["tcgen05", "mma_sync"])
def test_query_matches_numpy_forward(ctx, form):
    torch = pytest.importorskip("torch")
    from tressfx_gb300.api import NeuralSDF
    lo, hi = np.array([-0.2, 1.3, -0.25]), np.array([0.25, 1.8, 0.2])
    nsdf = NeuralSDF(ctx, lo, hi, cell_size=0.004, pose_scale=1.0 / 0.7, seed=3, max_samples=512, max_eval_samples=0)
    rng = np.random.default_rng(0)
    p = nsdf.params()
    nz = p != 0
    p[nz] *= rng.uniform(0.5, 1.5, nz.sum()).astype(np.float32)
    for a, b in ((R.P_B1, R.P_W2), (R.P_B2, R.P_W3), (R.P_B3, R.P_W4), (R.P_B4, R.P_W5)):
        p[a:b] = rng.normal(0, 0.3, b - a)
    p[R.P_B5] = 0.7
    nsdf.set_params(p)
    nsdf.set_inference(form)
    P = 3000
    pts = rng.uniform(lo, hi, (P, 3)).astype(np.float32)
    pose = (0.3, -0.45, 0.6)
    dev = torch.zeros((P, 4), dtype=torch.float32, device="cuda")
    dev[:, :3] = torch.from_numpy(pts).cuda()
    out = torch.empty(P, dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    nsdf.query_device(dev.data_ptr(), P, pose, out.data_ptr())
    ctx.synchronize()
    got = out.cpu().numpy() / np.float32(0.004)
    want = R.forward(p, R.features(pts, pose, R.frame(lo, hi, 1.0 / 0.7)))
    err = np.abs(got - want)
    assert np.isfinite(got).all()
    # bf16 activations: a one-ulp difference in an activation (different summation order, the
    # hardware tanh) moves the output by ~2^-8 of its scale
    assert err.max() < 0.05 + 0.03 * np.abs(want).max(), (err.max(), np.abs(want).max())
    assert np.median(err) < 0.01 + 0.006 * np.abs(want).max()
    nsdf.close()


def test_tcgen05_and_mma_sync_forward_agree(ctx):
    """The two forward passes of one network on 100,003 points (a ragged last tile): the same bf16
    network, so they differ only where accumulation order or the bias's extra bits move an activation
    by an ulp."""
    torch = pytest.importorskip("torch")
    from tressfx_gb300.api import NeuralSDF
    lo, hi = np.array([-0.2, 1.3, -0.25]), np.array([0.25, 1.8, 0.2])
    nsdf = NeuralSDF(ctx, lo, hi, cell_size=0.004, pose_scale=1.0 / 0.7, seed=5, max_samples=512, max_eval_samples=0)
    rng = np.random.default_rng(1)
    p = nsdf.params()
    for a, b in ((R.P_B1, R.P_W2), (R.P_B2, R.P_W3), (R.P_B3, R.P_W4), (R.P_B4, R.P_W5)):
        p[a:b] = rng.normal(0, 0.3, b - a)
    nsdf.set_params(p)
    P = 100003
    pts = rng.uniform(lo, hi, (P, 3)).astype(np.float32)
    dev = torch.zeros((P, 4), dtype=torch.float32, device="cuda")
    dev[:, :3] = torch.from_numpy(pts).cuda()
    outs = []
    for form in (1, 0):
        out = torch.full((P,), float("nan"), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        nsdf.set_inference(form)
        nsdf.query_device(dev.data_ptr(), P, (0.1, 0.2, -0.3), out.data_ptr())
        ctx.synchronize()
        outs.append(out.cpu().numpy() / np.float32(0.004))
    tc, ms = outs
    assert np.isfinite(tc).all() and np.isfinite(ms).all()
    scale = np.abs(ms).max()
    err = np.abs(tc - ms)
    assert err.max() < 0.03 * scale + 0.05, (err.max(), scale)
    assert np.median(err) < 0.003 * scale + 0.005, (np.median(err), scale)
    nsdf.close()


def test_training_step_matches_numpy_backward(ctx):
    """One training step on samples the test chooses: the weight and bias gradients of every layer
    (k_nsdf_train's backward pass, k_nsdf_wgrad's sums) against a NumPy backward pass of the same bf16
    network on the same drawn samples, the loss, and Adam's first step (k_nsdf_adam) on the GPU's own
    gradient."""
    from tressfx_gb300.api import NeuralSDF
    lo, hi = np.array([-0.2, 1.3, -0.25]), np.array([0.25, 1.8, 0.2])
    seed, pool, batch, lr = 11, 1000, 512, 1e-3
    nsdf = NeuralSDF(ctx, lo, hi, cell_size=0.004, pose_scale=1.0 / 0.7, seed=seed, max_samples=4096, max_eval_samples=0)
    rng = np.random.default_rng(4)
    p = nsdf.params()
    for a, b in ((R.P_B1, R.P_W2), (R.P_B2, R.P_W3), (R.P_B3, R.P_W4), (R.P_B4, R.P_W5)):
        p[a:b] = rng.normal(0, 0.3, b - a)
    p[R.P_B5] = 0.2
    nsdf.set_params(p)
    samples = np.zeros((pool, 8), np.float32)
    samples[:, :3] = rng.uniform(lo, hi, (pool, 3))
    samples[:, 3] = rng.uniform(-3.0, 3.0, pool)
    samples[:, 4:7] = rng.uniform(-0.6, 0.6, (pool, 3))
    samples[:, 7] = rng.uniform(0.5, 1.5, pool)
    nsdf.set_samples(0, samples)
    mean_loss = nsdf.train(1, batch=batch, lr=lr)
    g_gpu = nsdf.gradients()
    p1 = nsdf.params()
    drawn = R.drawn_samples(seed, 1, batch, pool)
    g_np, loss_np = R.train_gradients(p, samples[drawn], R.frame(lo, hi, 1.0 / 0.7))
    # the forward passes differ in the hardware tanh and sine: a bf16 ulp in some activations
    assert abs(mean_loss - loss_np / batch) < 0.02 * loss_np / batch, (mean_loss, loss_np / batch)
    blocks = {"W1": (R.P_W1, R.P_B1), "b1": (R.P_B1, R.P_W2), "W2": (R.P_W2, R.P_B2), "b2": (R.P_B2, R.P_W3),
              "W3": (R.P_W3, R.P_B3), "b3": (R.P_B3, R.P_W4), "W4": (R.P_W4, R.P_B4), "b4": (R.P_B4, R.P_W5),
              "W5": (R.P_W5, R.P_B5), "b5": (R.P_B5, R.NPARAM)}
    for name, (a, b) in blocks.items():
        x, y = g_gpu[a:b].astype(np.float64), g_np[a:b].astype(np.float64)
        ny = np.linalg.norm(y)
        assert ny > 0, name
        rel = np.linalg.norm(x - y) / ny
        cos = float(x @ y / (np.linalg.norm(x) * ny))
        assert rel < 0.05 and cos > 0.998, (name, rel, cos)
    # Adam's first step at this call's learning rate (the cosine schedule at step 0 of 1)
    f = np.float32
    lr0 = f(lr) * (f(0.1) + f(0.45) * (f(1.0) + f(1.0)))
    want = R.adam_first_step(p, g_gpu, lr0)
    np.testing.assert_allclose(p1, want, rtol=2e-6, atol=1e-9)
    nsdf.close()


@pytest.fixture(scope="module")
def small_proxy(ctx):
    from tressfx_gb300 import synthetic as S
    from tressfx_gb300.neural import train_proxy
    sc = S.scene_neural(num_guides=500, n=16, triangles=3000, sdf_cells=48, frames=12)
    nsdf, rep = train_proxy(ctx, sc.objects[0], poses=96, samples_per_pose=4096, eval_poses=8,
                            eval_samples_per_pose=4096, steps=1500, batch=4096, lr=2e-3, contact_slack_cells=2.0)
    print("proxy:", rep)
    yield sc, nsdf, rep
    nsdf.close()


def test_training_learns_the_grid_sdf(small_proxy):
    _, _, rep = small_proxy
    assert rep.samples == 96 * 4096 and rep.eval_points > 1000
    assert math.isfinite(rep.final_loss) and rep.final_loss < 0.5
    assert rep.error_mean_cells < 0.5, rep


def test_collision_through_the_proxy_matches_the_grid(ctx, small_proxy):
    """Vertices the network places outside the contact band are not collided; the band is collided
    exactly on the grid.  With the network within the slack of the grid, every buffer equals the
    grid-collided frames bit for bit, and the band is a strict subset of the vertices."""
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.headless import NeuralPipeline, PlainPipeline
    sc, nsdf, _ = small_proxy
    a = PlainPipeline(ctx, sc)
    b = NeuralPipeline(ctx, sc, nsdf)
    try:
        for f in range(10):
            a.step(f)
            fin = b.step(f) if f < 9 else None
            if f == 9:
                from tressfx_gb300.headless import FrameInputs
                fin = FrameInputs(sc, f)
                b.prepare(fin)
                b.run(fin, record_band=True)
        band = b.band_counts[-1]
        total = b.hair[0].num_vertices
        for buf in (A.BUF_POSITIONS, A.BUF_POSITIONS_PREV, A.BUF_TANGENTS):
            x, y = a.hair[0].read(buf).view(np.uint32), b.hair[0].read(buf).view(np.uint32)
            assert np.array_equal(x, y), f"buffer {buf}: {int((x != y).any(axis=1).sum())} vertices differ"
        assert 0 < band < total
    finally:
        a.close()
        b.close()


def _gated_grid_check(ctx, sc, nsdf, frames_before: int):
    """Runs a proxy frame up to its collision, recomputes the contact band on the host from the
    network's own outputs (tfx_nsdf_query on the same positions) and returns the proxy path's grid, the
    full grid of the same pose and the cells the band's lookups read (vertices whose output lies within
    1e-3 cells of the band's edge are left out, as rounding could put them on either side)."""
    import torch
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.api import SDFCollision
    from tressfx_gb300.headless import FrameInputs, NeuralPipeline
    from tressfx_gb300.synthetic import margin_world
    obj = sc.objects[0]
    b = NeuralPipeline(ctx, sc, nsdf)
    cells = int(np.prod(obj.sdf_dims))
    full = SDFCollision(ctx, cells)
    full.bind_mesh(b.meshes[0])
    try:
        for f in range(frames_before):
            b.step(f)
        fin = FrameInputs(sc, frames_before)
        b.prepare(fin)
        b.meshes[0].skin(fin.mesh_bones[0])      # NeuralPipeline.run up to the collision
        b.sim.simulate(b.hair)
        h, g = b.hair[0], fin.grids[0]
        pose = sc.meta["pose_fn"](frames_before * sc.dt)
        P = h.read(A.BUF_POSITIONS).reshape(-1, 4)
        pos_ptr, _ = h.device_buffer(A.BUF_POSITIONS)
        out = torch.empty(len(P), dtype=torch.float32, device="cuda")
        torch.cuda.synchronize()
        nsdf.query_device(pos_ptr, len(P), pose, out.data_ptr())
        torch.cuda.synchronize()
        y = out.cpu().numpy() / np.float32(nsdf.cell_size)   # the query returns world units, the band is in cells
        m = margin_world(obj, g)
        limit = np.float32(np.float32(m) / np.float32(nsdf.cell_size)) + np.float32(2.0)
        j = np.arange(len(P)) % h.n
        sure = (j >= 2) & (y < limit - np.float32(1e-3))
        band = nsdf.collide(h, b.sdfs[0], g, m, pose, band=True)
        full.update(g)
        gated, want = b.sdfs[0].read(cells), full.read(cells)
        o = np.array([g.origin[0], g.origin[1], g.origin[2]], np.float32)
        q = np.trunc((P[sure, :3].astype(np.float32) - o) / np.float32(g.cell_size)).astype(np.int64)
        nx, ny, nz = obj.sdf_dims
        idx = set()
        for d in np.stack(np.meshgrid(range(3), range(3), range(3), indexing="ij"), -1).reshape(-1, 3):
            c = q + d
            ok = (c >= 0).all(1) & (c[:, 0] < nx) & (c[:, 1] < ny) & (c[:, 2] < nz)
            idx.update(((c[ok, 2] * ny + c[ok, 1]) * nx + c[ok, 0]).tolist())
        return gated, want, np.array(sorted(idx), np.int64), int(sure.sum()), band
    finally:
        full.close()
        b.close()


def test_gated_grid_is_exact_at_the_band_cells(ctx, small_proxy):
    """The proxy path builds the grid only at the cells its contact band's lookups read; there every
    word equals the full build's, whatever triangles the coarse 4x4x4-cell map let it skip."""
    sc, nsdf, _ = small_proxy
    gated, want, idx, sure, band = _gated_grid_check(ctx, sc, nsdf, 6)
    assert sure > 0 and band >= sure and len(idx) > 0
    bad = idx[gated[idx] != want[idx]]
    assert len(bad) == 0, f"{len(bad)} of {len(idx)} band cells differ"


@pytest.fixture(scope="module")
def grid128_proxy(ctx):
    """The proxy workload's head mesh (20k triangles) and 128^3 grid, with fewer guides, and a proxy
    trained briefly (the band is then wider, which the check only welcomes)."""
    from tressfx_gb300 import synthetic as S
    from tressfx_gb300.neural import train_proxy
    sc = S.scene_neural(num_guides=5000, n=32, frames=12)
    nsdf, rep = train_proxy(ctx, sc.objects[0], poses=64, samples_per_pose=4096, eval_poses=4,
                            eval_samples_per_pose=4096, steps=1500, batch=4096, lr=3e-3, contact_slack_cells=2.0)
    yield sc, nsdf, rep
    nsdf.close()


def test_gated_grid_is_exact_at_the_band_cells_128(ctx, grid128_proxy):
    sc, nsdf, _ = grid128_proxy
    gated, want, idx, sure, band = _gated_grid_check(ctx, sc, nsdf, 6)
    assert sure > 0 and band >= sure and len(idx) > 0
    bad = idx[gated[idx] != want[idx]]
    assert len(bad) == 0, f"{len(bad)} of {len(idx)} band cells differ"


def test_pose_outside_training_range_takes_the_grid_path(ctx, small_proxy):
    """A pose outside the range the proxy was trained on: every vertex is collided on the full grid,
    so the frames equal the grid-collided ones bit for bit and the band reports every vertex."""
    from tressfx_gb300 import _capi as A
    from tressfx_gb300.headless import FrameInputs, NeuralPipeline, PlainPipeline
    sc, nsdf, _ = small_proxy
    pose_fn = sc.meta["pose_fn"]
    sc.meta["pose_fn"] = lambda t: (2.5, -2.5, 2.5)   # radians, far outside the +-40 degree training poses
    a = PlainPipeline(ctx, sc)
    b = NeuralPipeline(ctx, sc, nsdf)
    try:
        for f in range(6):
            a.step(f)
            fin = FrameInputs(sc, f)
            b.prepare(fin)
            b.run(fin, record_band=True)
        assert b.band_counts[-1] == b.hair[0].num_vertices
        for buf in (A.BUF_POSITIONS, A.BUF_POSITIONS_PREV, A.BUF_TANGENTS):
            x, y = a.hair[0].read(buf).view(np.uint32), b.hair[0].read(buf).view(np.uint32)
            assert np.array_equal(x, y), f"buffer {buf}"
    finally:
        sc.meta["pose_fn"] = pose_fn
        a.close()
        b.close()
