"""Differentiable leaf shading (svo_diff_forward / svo_diff_backward) against
the FP64 host oracle (oracle/diff_oracle.py) fed with the CPU raymarch's hit
buffers: forward colours, analytic gradients, and central finite differences
(h = 1e-3, Richardson-extrapolated with h/2) on 256 random leaves to 1e-4
relative.  The torch.autograd.Function
below exists only in this test harness."""
import numpy as np
import pytest

import diff_oracle

pytestmark = pytest.mark.gpu

REL_TOL = 1e-4


def make_function(torch):
    class SvoShade(torch.autograd.Function):
        @staticmethod
        def forward(ctx, leaf_rgb, leaf_normal, tree, rays, W, H, V, lights, retrace):
            R = W * H * V
            rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
            hit = None if retrace else torch.empty(R, dtype=torch.int32, device="cuda")
            tree.diff_forward(rays, W, H, V, lights, leaf_rgb, leaf_normal, rgb, hit_leaf=hit)
            ctx.save_for_backward(leaf_rgb, leaf_normal)
            ctx.extra = (tree, rays, W, H, V, lights, hit)
            return rgb

        @staticmethod
        def backward(ctx, g):
            leaf_rgb, leaf_normal = ctx.saved_tensors
            tree, rays, W, H, V, lights, hit = ctx.extra
            gr = torch.zeros_like(leaf_rgb)
            gn = torch.zeros_like(leaf_normal)
            tree.diff_backward(rays, W, H, V, lights, leaf_rgb, leaf_normal, g.contiguous(), gr, gn, hit_leaf=hit)
            return gr, gn, None, None, None, None, None, None, None

    return SvoShade


@pytest.fixture(scope="module")
def problem(cuda, svo, oracle, scenes):
    torch = cuda
    grid = scenes.sphere_scene(128, 20, 7)
    tree = svo.VoxelOctree(svo.VoxelData(grid))
    words = tree.words()
    center = tree.center()
    W, H = 96, 64
    cams = scenes.orbit_cameras(3, 11, center, radius=1.6)
    rays = np.concatenate([scenes.camera_rays(c, W, H) for c in cams])
    lights = np.stack([scenes.headlight(c) for c in cams]).astype(np.float32)
    V = len(cams)
    rng = np.random.default_rng(3)
    nw = words.size
    p_rgb = rng.random((nw, 3), dtype=np.float32)
    p_n = rng.random((nw, 3), dtype=np.float32)
    target = rng.random((rays.shape[0], 3)).astype(np.float32)
    # the CPU raymarch's hit buffer (the reference's leaf for every ray)
    ref = oracle.raymarch(words, rays, threads=4)
    leaf = np.where(ref["hit"] == 1, ref["leaf"], np.uint32(0xFFFFFFFF)).astype(np.uint32)
    ray_light = np.repeat(lights, W * H, axis=0)
    return dict(tree=tree, words=words, W=W, H=H, V=V, rays=rays, lights=lights, p_rgb=p_rgb, p_n=p_n,
                target=target, leaf=leaf, ray_light=ray_light, w=1.0 / (3 * rays.shape[0]))


def _device(torch, pb):
    return (torch.from_numpy(pb["rays"]).cuda(), torch.from_numpy(pb["lights"]).cuda(),
            torch.from_numpy(pb["p_rgb"]).cuda().requires_grad_(), torch.from_numpy(pb["p_n"]).cuda().requires_grad_(),
            torch.from_numpy(pb["target"]).cuda())


def _gpu_grads(torch, svo, pb, retrace=False):
    Fn = make_function(torch)
    rays, lights, p_rgb, p_n, target = _device(torch, pb)
    rgb = Fn.apply(p_rgb, p_n, pb["tree"], rays, pb["W"], pb["H"], pb["V"], lights, retrace)
    loss = (pb["w"] * (rgb - target) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    return rgb.detach().cpu().numpy(), p_rgb.grad.cpu().numpy(), p_n.grad.cpu().numpy(), float(loss.item())


def _rel_err(a, b, floor):
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def _leaf_rel_err(g, ref):
    """Per-leaf relative error of the 3-vector gradient, ||g - ref|| / ||ref||,
    over leaves whose gradient is at least 1e-3 of the largest (below that an
    FP32 sum of cancelling per-ray terms has no relative accuracy left)."""
    num = np.linalg.norm(g - ref, axis=-1)
    den = np.linalg.norm(ref, axis=-1)
    keep = den >= 1e-3 * den.max()
    return num[keep] / den[keep], keep

def test_forward_matches_fp64_oracle(cuda, svo, problem):
    torch = cuda
    pb = problem
    rays, lights, p_rgb, p_n, _ = _device(torch, pb)
    R = rays.shape[0]
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    hit = torch.empty(R, dtype=torch.int32, device="cuda")
    pb["tree"].diff_forward(rays, pb["W"], pb["H"], pb["V"], lights, p_rgb.detach(), p_n.detach(), rgb, hit_leaf=hit)
    torch.cuda.synchronize()
    assert np.array_equal(hit.cpu().numpy().view(np.uint32), pb["leaf"])  # traversal unchanged
    ref = diff_oracle.shade(pb["leaf"], pb["rays"][:, 3:], pb["ray_light"], pb["p_rgb"], pb["p_n"])
    assert np.max(np.abs(rgb.cpu().numpy() - ref)) < 2e-6
    assert (pb["leaf"] != 0xFFFFFFFF).mean() > 0.1


def test_adjoint_matches_fp64_gradient(cuda, svo, problem):
    torch = cuda
    pb = problem
    _, g_rgb, g_n, loss = _gpu_grads(torch, svo, pb)
    ref_loss = diff_oracle.loss(pb["leaf"], pb["rays"][:, 3:], pb["ray_light"], pb["p_rgb"], pb["p_n"], pb["target"],
                                pb["w"])
    assert abs(loss - ref_loss) <= 1e-5 * abs(ref_loss)
    r_rgb, r_n = diff_oracle.gradient(pb["leaf"], pb["rays"][:, 3:], pb["ray_light"], pb["p_rgb"], pb["p_n"],
                                      pb["target"], pb["w"], pb["words"].size)
    hit = np.unique(pb["leaf"][pb["leaf"] != 0xFFFFFFFF]).astype(np.int64)
    for gpu, ref in ((g_rgb, r_rgb), (g_n, r_n)):
        floor = 1e-3 * np.abs(ref[hit]).max()
        assert np.max(_rel_err(gpu[hit], ref[hit], floor)) < REL_TOL
    # parameters of leaves no ray hits get no gradient
    miss = np.setdiff1d(np.arange(pb["words"].size), hit)
    assert not g_rgb[miss].any() and not g_n[miss].any()


def test_adjoint_matches_finite_differences(cuda, svo, problem):
    torch = cuda
    pb = problem
    _, g_rgb, g_n, _ = _gpu_grads(torch, svo, pb)
    hit = np.unique(pb["leaf"][pb["leaf"] != 0xFFFFFFFF])
    leaves = np.random.default_rng(5).choice(hit, size=256, replace=False)
    fd_rgb, fd_n, kink = diff_oracle.finite_differences(pb["leaf"], pb["rays"][:, 3:], pb["ray_light"], pb["p_rgb"],
                                                        pb["p_n"], pb["target"], pb["w"], leaves, h=1e-3,
                                                        richardson=True)
    li = leaves.astype(np.int64)
    err, keep = _leaf_rel_err(g_rgb[li], fd_rgb)
    assert keep.mean() > 0.9 and err.max() < REL_TOL
    # leaves where a +-h step of some normal component crosses a kink of
    # |l.n| or max(l.r, 0) (the loss is not differentiable there) are left out
    smooth = ~kink.any(axis=1)
    assert smooth.mean() > 0.8
    err, keep = _leaf_rel_err(g_n[li][smooth], fd_n[smooth])
    assert keep.mean() > 0.9 and err.max() < REL_TOL


def test_retrace_mode_matches_recorded_mode(cuda, svo, problem):
    torch = cuda
    a = _gpu_grads(torch, svo, problem, retrace=False)
    b = _gpu_grads(torch, svo, problem, retrace=True)
    assert np.array_equal(a[0], b[0])
    for x, y in zip(a[1:3], b[1:3]):
        np.testing.assert_allclose(x, y, rtol=1e-5, atol=1e-12)


def test_adam_reduces_loss(cuda, svo, problem):
    torch = cuda
    pb = problem
    Fn = make_function(torch)
    rays, lights, p_rgb, p_n, _ = _device(torch, pb)
    # targets rendered from ground-truth parameters, so the loss can reach 0
    rng = np.random.default_rng(9)
    gt_rgb = torch.from_numpy(rng.random(pb["p_rgb"].shape, dtype=np.float32)).cuda()
    gt_n = torch.from_numpy(rng.random(pb["p_n"].shape, dtype=np.float32)).cuda()
    target = torch.empty((rays.shape[0], 3), dtype=torch.float32, device="cuda")
    pb["tree"].diff_forward(rays, pb["W"], pb["H"], pb["V"], lights, gt_rgb, gt_n, target)
    opt = torch.optim.Adam([p_rgb, p_n], lr=1e-2)
    losses = []
    for _ in range(60):
        opt.zero_grad()
        rgb = Fn.apply(p_rgb, p_n, pb["tree"], rays, pb["W"], pb["H"], pb["V"], lights, False)
        loss = (pb["w"] * (rgb - target) ** 2).sum()
        loss.backward()
        opt.step()
        losses.append(loss.item())
    assert losses[-1] < 0.5 * losses[0]


def test_leaf_adam_matches_torch_adam(cuda, svo):
    torch = cuda
    gen = torch.Generator(device="cuda").manual_seed(3)
    shapes = [(1000003, 3), (7,)]  # a vectorised body with a scalar tail, and a tiny tensor
    ps = [torch.rand(s, generator=gen, device="cuda") for s in shapes]
    ref = [p.clone().requires_grad_() for p in ps]
    mine = [p.clone() for p in ps]
    opt_ref = torch.optim.Adam(ref, lr=1e-2)
    opt = svo.LeafAdam(mine, lr=1e-2)
    for step in range(6):
        grads = [torch.randn(s, generator=gen, device="cuda") * (1 + step) for s in shapes]
        for r, g in zip(ref, grads):
            r.grad = g.clone()
        for m, g in zip(mine, grads):
            m.grad = g.clone()
        opt_ref.step()
        opt.step()
        torch.cuda.synchronize()
        for r, m in zip(ref, mine):
            torch.testing.assert_close(m, r.detach(), rtol=2e-6, atol=2e-7)
            assert not m.grad.any()  # zeroed in the same pass
