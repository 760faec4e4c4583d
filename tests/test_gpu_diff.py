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


def test_fused_l2_adjoint_matches_unfused(cuda, svo, problem):
    """svo_diff_backward_l2 (the loss gradient formed in the kernel) against
    svo_diff_backward fed with dL/drgb from torch; its loss sum, and its
    record of touched leaves against the hit leaves."""
    torch = cuda
    pb = problem
    rays, lights, p_rgb, p_n, target = _device(torch, pb)
    R = rays.shape[0]
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    hit = torch.empty(R, dtype=torch.int32, device="cuda")
    args = (rays, pb["W"], pb["H"], pb["V"], lights, p_rgb.detach(), p_n.detach())
    pb["tree"].diff_forward(*args, rgb, hit_leaf=hit)
    scale = 2.0 * pb["w"]
    d_rgb = (rgb - target) * scale
    g1 = [torch.zeros_like(p_rgb), torch.zeros_like(p_n)]
    pb["tree"].diff_backward(*args, d_rgb, g1[0], g1[1], hit_leaf=hit)
    g2 = [torch.zeros_like(p_rgb), torch.zeros_like(p_n)]
    loss_sum = torch.zeros(1, dtype=torch.float64, device="cuda")
    leaves = svo.LeafSet(pb["words"].size)
    pb["tree"].diff_backward_l2(*args, rgb, target, scale, g2[0], g2[1], hit_leaf=hit, loss_sum=loss_sum,
                                leaves=leaves)
    # the re-traced form gives the same gradients and adds nothing new to the record
    g3 = [torch.zeros_like(p_rgb), torch.zeros_like(p_n)]
    pb["tree"].diff_backward_l2(*args, rgb, target, scale, g3[0], g3[1], leaves=leaves)
    torch.cuda.synchronize()
    for a, b, c in zip(g1, g2, g3):
        torch.testing.assert_close(b, a, rtol=1e-5, atol=1e-12)
        torch.testing.assert_close(c, a, rtol=1e-5, atol=1e-12)
    ref_loss = float(((rgb.double() - target.double()) ** 2).sum().item())
    assert abs(loss_sum.item() - ref_loss) <= 1e-5 * ref_loss
    hit_leaves = np.unique(pb["leaf"][pb["leaf"] != 0xFFFFFFFF])
    listed = leaves.list[:leaves.size()].cpu().numpy().view(np.uint32)
    assert np.array_equal(np.sort(listed), hit_leaves)
    bits = leaves.touched.cpu().numpy().view(np.uint32)
    on = np.nonzero((bits[:, None] >> np.arange(32, dtype=np.uint32)) & 1)
    assert np.array_equal(np.sort(on[0] * 32 + on[1]), hit_leaves)


def test_sparse_adam_equals_dense_adam(cuda, svo, problem):
    """Adam over the touched leaves only (svo_adam_step_leaves) gives the
    dense svo_adam_step's parameters bit for bit, step after step: leaves
    never touched keep zero moments, which the dense update leaves alone."""
    torch = cuda
    pb = problem
    rays, lights, p0_rgb, p0_n, target = _device(torch, pb)
    dense = [p0_rgb.detach().clone(), p0_n.detach().clone()]
    sparse = [p0_rgb.detach().clone(), p0_n.detach().clone()]
    leaves = svo.LeafSet(pb["words"].size)
    opt_d = svo.LeafAdam(dense, lr=1e-2)
    opt_s = svo.LeafAdam(sparse, lr=1e-2, leaves=leaves)
    R = rays.shape[0]
    rgb = torch.empty((R, 3), dtype=torch.float32, device="cuda")
    hit = torch.empty(R, dtype=torch.int32, device="cuda")
    # the views change every step, so the record grows over the steps
    n_pix = pb["W"] * pb["H"]
    for step in range(6):
        v = step % pb["V"]
        sl = slice(v * n_pix, (v + 1) * n_pix)
        g = [torch.zeros_like(dense[0]), torch.zeros_like(dense[1])]
        args = (rays[sl], pb["W"], pb["H"], 1, lights[v:v + 1], dense[0], dense[1])
        pb["tree"].diff_forward(*args, rgb[sl], hit_leaf=hit[sl])
        pb["tree"].diff_backward_l2(*args, rgb[sl], target[sl], 2.0 * pb["w"], g[0], g[1], hit_leaf=hit[sl],
                                    leaves=leaves)
        for p, gp in zip(dense, g):
            p.grad = gp
        for p, gp in zip(sparse, g):
            p.grad = gp.clone()
        opt_d.step()
        opt_s.step()
        torch.cuda.synchronize()
        for a, b in zip(dense, sparse):
            assert torch.equal(a.view(torch.int32), b.view(torch.int32)), step
        for (m1, v1), (m2, v2) in zip(opt_d.state, opt_s.state):
            assert torch.equal(m1, m2) and torch.equal(v1, v2), step
        assert not sparse[0].grad.any() and not sparse[1].grad.any()
    assert 0 < leaves.size() < pb["words"].size


def test_leaf_records_match_separate_arrays(cuda, svo, problem):
    """The 8-float leaf record layout (rgb at 0..2, normal at 3..5, through
    the *_stride entry points) against the two 3-float arrays: the same
    colours and hit leaves bit for bit, the same gradients up to the order of
    the atomic sums, and Adam over whole records (width 8) gives the same
    parameters while the two unused floats stay as they are."""
    torch = cuda
    pb = problem
    rays, lights, p_rgb, p_n, target = _device(torch, pb)
    p_rgb, p_n = p_rgb.detach(), p_n.detach()
    nw = p_rgb.shape[0]
    rec = torch.full((nw, 8), 7.0, dtype=torch.float32, device="cuda")
    rec[:, 0:3] = p_rgb
    rec[:, 3:6] = p_n
    R = rays.shape[0]
    geo = (rays, pb["W"], pb["H"], pb["V"], lights)
    rgb3, rgb8 = (torch.empty((R, 3), dtype=torch.float32, device="cuda") for _ in range(2))
    hit3, hit8 = (torch.empty(R, dtype=torch.int32, device="cuda") for _ in range(2))
    pb["tree"].diff_forward(*geo, p_rgb, p_n, rgb3, hit_leaf=hit3)
    pb["tree"].diff_forward(*geo, rec[:, 0:3], rec[:, 3:6], rgb8, hit_leaf=hit8, param_stride=8)
    torch.cuda.synchronize()
    assert torch.equal(rgb3.view(torch.int32), rgb8.view(torch.int32)) and torch.equal(hit3, hit8)
    scale = 2.0 * pb["w"]
    g3 = [torch.zeros_like(p_rgb), torch.zeros_like(p_n)]
    grec = torch.zeros_like(rec)
    leaves3, leaves8 = svo.LeafSet(nw), svo.LeafSet(nw)
    pb["tree"].diff_backward_l2(*geo, p_rgb, p_n, rgb3, target, scale, g3[0], g3[1], hit_leaf=hit3, leaves=leaves3)
    pb["tree"].diff_backward_l2(*geo, rec[:, 0:3], rec[:, 3:6], rgb8, target, scale, grec[:, 0:3], grec[:, 3:6],
                                hit_leaf=hit8, leaves=leaves8, param_stride=8)
    # the plain adjoint with dL/drgb from torch, in records too
    grec2 = torch.zeros_like(rec)
    pb["tree"].diff_backward(*geo, rec[:, 0:3], rec[:, 3:6], (rgb8 - target) * scale, grec2[:, 0:3],
                             grec2[:, 3:6], hit_leaf=hit8, param_stride=8)
    torch.cuda.synchronize()
    torch.testing.assert_close(grec[:, 0:3], g3[0], rtol=1e-5, atol=1e-12)
    torch.testing.assert_close(grec[:, 3:6], g3[1], rtol=1e-5, atol=1e-12)
    torch.testing.assert_close(grec2[:, 0:6], grec[:, 0:6], rtol=1e-5, atol=1e-12)
    assert not grec[:, 6:].any()
    assert leaves8.size() == leaves3.size()
    # one sparse Adam step each, from the same gradients
    sep = [p_rgb.clone(), p_n.clone()]
    sep[0].grad, sep[1].grad = grec[:, 0:3].contiguous(), grec[:, 3:6].contiguous()
    rec.grad = grec
    svo.LeafAdam(sep, lr=1e-2, leaves=leaves3).step()
    svo.LeafAdam([rec], lr=1e-2, leaves=leaves8, width=8).step()
    torch.cuda.synchronize()
    assert torch.equal(rec[:, 0:3].contiguous().view(torch.int32), sep[0].view(torch.int32))
    assert torch.equal(rec[:, 3:6].contiguous().view(torch.int32), sep[1].view(torch.int32))
    assert bool((rec[:, 6:] == 7.0).all())
    with pytest.raises(Exception):
        pb["tree"].diff_forward(*geo, p_rgb, p_n, rgb3, param_stride=2)
