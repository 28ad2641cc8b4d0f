"""Adjoint of the textured resolve (an addition): the GPU forward and the
hand-written GPU backward, through the C ABI, against
  - a float64 CPU reference of the same shading and its exact gradient,
  - central finite differences (h = 1e-3) of the float64 loss on 200 seeded
    parameters, at fixed visibility,
and wrapped in a torch.autograd.Function (test harness only)."""
import numpy as np
import pytest
import torch

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi, diff, scene
from vk_gltf_viewer_gb300.renderer import DeviceScene

pytestmark = pytest.mark.gpu

W = H = 96
NVIEWS = 4


class Setup:
    def __init__(self, level=3, tex=64, seed=5):
        rng = np.random.default_rng(seed)
        self.mesh = scene.icosphere(level)
        nv = self.mesh.positions.shape[0]
        self.colors = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
        self.texture = rng.uniform(0, 1, size=(tex, tex, 3)).astype(np.float32)
        self.scene = diff.DiffScene.create(self.mesh, self.colors, self.texture)
        self.cams = []
        for _ in range(NVIEWS):
            v = rng.normal(size=3)
            eye = 3.0 * v / np.linalg.norm(v)
            self.cams.append(scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, W / H))
        self.views = [diff.DiffViewBuffers.allocate(W, H, c) for c in self.cams]
        # targets: perturbed positions and a separately seeded texture
        trng = np.random.default_rng(seed + 100)
        pos_t = self.mesh.positions + trng.normal(0, 0.01, size=self.mesh.positions.shape).astype(np.float32)
        tex_t = trng.uniform(0, 1, size=self.texture.shape).astype(np.float32)
        self.target_scene = diff.DiffScene.create(self.mesh, self.colors, tex_t, positions=pos_t)
        self.scale = 1.0 / (3 * W * H * NVIEWS)
        self._ids = None

    def render(self, r, sc=None):
        out = [torch.zeros(W * H * 3, device="cuda") for _ in self.views]
        diff.forward(r, sc or self.scene, self.views, out)
        torch.cuda.synchronize()
        self._ids = None
        return out

    def ids_of(self, v):
        """Visibility ids of the last render (cached per render)."""
        if self._ids is None:
            self._ids = {id(x): x.ids() for x in self.views}
        return self._ids[id(v)]

    @staticmethod
    def host_target(t):
        return t.cpu().numpy() if torch.is_tensor(t) else t


@pytest.fixture(scope="module")
def su(renderer):
    return Setup()


def vp_of(cam):
    return np.frombuffer(bytes(cam), np.float32)[32:48].copy()


def test_visibility_is_the_raster_of_the_oracle(renderer, su):
    su.render(renderer)
    host = scene.HostScene(meshes=[su.mesh], prim_materials=[1],
                           materials=np.concatenate([scene.default_material(), scene.make_material()]),
                           transforms=scene.to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])
    osc = ob.OracleScene(host)
    for v, cam in zip(su.views, su.cams):
        exp = ob.frame(osc, cam, W, H, 0)["ids"]
        assert np.array_equal(su.ids_of(v), exp)


def _moved(mesh, pos):
    """The mesh with new vertex positions (same meshlets, no cones)."""
    import dataclasses
    verts = mesh.vertices.copy()
    verts["position"] = pos
    return dataclasses.replace(mesh, vertices=verts, positions=pos, cones=None)


@pytest.mark.parametrize("mode", [1, 2])
def test_cone_culled_passes_keep_the_visibility(renderer, su, mode):
    """The visibility passes with meshlet normal cones rebuilt from the
    current positions (forced on) or without them (forced off) give the
    oracle's unculled raster, at the stored and at perturbed positions."""
    rng = np.random.default_rng(17)
    for pos in (su.mesh.positions, su.mesh.positions + rng.normal(0, 0.02, size=su.mesh.positions.shape)):
        pos = np.ascontiguousarray(pos, np.float32)
        mesh = _moved(su.mesh, pos)
        host = scene.HostScene(meshes=[mesh], prim_materials=[1],
                               materials=np.concatenate([scene.default_material(), scene.make_material()]),
                               transforms=scene.to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])
        osc = ob.OracleScene(host)
        sc = diff.DiffScene.create(su.mesh, su.colors, su.texture, positions=pos, cone_mode=mode)
        su.render(renderer, sc)
        for v, cam in zip(su.views, su.cams):
            assert np.array_equal(su.ids_of(v), ob.frame(osc, cam, W, H, 0)["ids"])
    su._ids = None


def test_forward_matches_float64(renderer, su):
    rgb = su.render(renderer)
    for v, cam, out in zip(su.views, su.cams, rgb):
        _, ref, _ = ob.diff_f64(su.mesh, su.mesh.positions, su.colors, su.mesh.uvs, su.texture, vp_of(cam), W, H,
                                su.ids_of(v), want_rgb=True)
        err = np.abs(out.cpu().numpy() - ref).max()
        assert err < 5e-4, err


def gpu_grads(renderer, su, targets):
    gp = torch.zeros_like(su.scene.positions)
    gc = torch.zeros_like(su.scene.colors)
    gt = torch.zeros_like(su.scene.texture)
    loss = torch.zeros(1, device="cuda")
    diff.backward(renderer, su.scene, su.views, gp, gc, gt, targets=targets, scale=su.scale, loss=loss)
    torch.cuda.synchronize()
    return float(loss.item()), gp.cpu().numpy().reshape(-1), gc.cpu().numpy().reshape(-1), gt.cpu().numpy().reshape(-1)


def f64_loss_and_grads(su, targets, positions=None, colors=None, texture=None, grads=True, cells=False):
    pos = su.mesh.positions if positions is None else positions
    col = su.colors if colors is None else colors
    tex = su.texture if texture is None else texture
    total, g, cs = 0.0, None, []
    for v, cam, t in zip(su.views, su.cams, targets):
        c = np.zeros(2 * W * H, np.int32) if cells else None
        loss, _, gg = ob.diff_f64(su.mesh, pos, col, su.mesh.uvs, tex, vp_of(cam), W, H, su.ids_of(v),
                                  target=su.host_target(t), scale=su.scale, want_grads=grads, cells=c)
        total += loss
        cs.append(c)
        if grads:
            g = gg if g is None else tuple(a + b for a, b in zip(g, gg))
    return (total, g, cs) if cells else (total, g)


def test_gradients_match_float64_reference(renderer, su):
    targets = su.render(renderer, su.target_scene)
    su.render(renderer)  # visibility of the current parameters
    loss, gp, gc, gt = gpu_grads(renderer, su, targets)
    ref_loss, (rp, rc, rt) = f64_loss_and_grads(su, targets)
    assert abs(loss - ref_loss) <= 1e-4 * abs(ref_loss)
    for name, g, r in (("positions", gp, rp), ("colors", gc, rc), ("texels", gt, rt)):
        rel = np.linalg.norm(g - r) / np.linalg.norm(r)
        assert rel < 1e-3, (name, rel)


def test_finite_differences_200_params(renderer, su):
    """Central differences with step h = 1e-3 of the float64 loss at fixed
    visibility against the GPU adjoint, on 200 seeded parameters with a
    non-zero gradient: 60 position, 60 colour and 80 texel coordinates.

    The loss is quadratic in colours and texels, so the two-point difference
    is exact there.  In positions it is rational (perspective barycentrics)
    and the two-point difference carries an O(h^2) truncation error that
    reaches a few percent at h = 1e-3 on triangles seen at grazing angles; the
    position check therefore uses the four-point central difference over
    {+-h, +-h/2} (Richardson: (4 D(h/2) - D(h)) / 3, error O(h^4)).
    Bilinear filtering has a derivative jump wherever a sample crosses a
    texel centre, so a position is only drawn when no pixel of any view
    changes bilinear cell across its stencil.  Parameters are drawn among
    those whose float64 gradient is at least 1e-3 of the largest of their
    kind (three quarters of each kind or more): a near-zero gradient is a
    sum of cancelling per-pixel terms whose fp32 rounding sets an absolute,
    not a relative, error floor."""
    targets = su.render(renderer, su.target_scene)
    su.render(renderer)
    _, gp, gc, gt = gpu_grads(renderer, su, targets)
    targets = [t.cpu().numpy() for t in targets]
    rng = np.random.default_rng(123)
    h = 1e-3
    base = {"pos": su.mesh.positions.astype(np.float64), "col": su.colors.astype(np.float64),
            "tex": su.texture.astype(np.float64)}
    grads = {"pos": gp, "col": gc, "tex": gt}
    _, ref64, cells0 = f64_loss_and_grads(su, targets, cells=True)
    ref64 = dict(zip(("pos", "col", "tex"), ref64))

    def loss_at(kind, i, step):
        arrs = {k: v.copy() for k, v in base.items()}
        arrs[kind].reshape(-1)[i] += step
        loss, _, cells = f64_loss_and_grads(su, targets, arrs["pos"], arrs["col"], arrs["tex"], grads=False,
                                            cells=True)
        return loss, all(np.array_equal(a, b) for a, b in zip(cells, cells0))

    errs, kinked = [], 0
    for kind, n in (("pos", 60), ("col", 60), ("tex", 80)):
        taken = 0
        mag = np.abs(ref64[kind])
        for i in rng.permutation(np.nonzero(mag >= 1e-3 * mag.max())[0]):
            if kind == "pos":
                (lp, s1), (lm, s2), (lp2, s3), (lm2, s4) = (loss_at(kind, i, s) for s in (h, -h, h / 2, -h / 2))
                if not (s1 and s2 and s3 and s4):
                    kinked += 1
                    continue
                fd = (4.0 * (lp2 - lm2) / h - (lp - lm) / (2 * h)) / 3.0
            else:
                fd = (loss_at(kind, i, h)[0] - loss_at(kind, i, -h)[0]) / (2 * h)
            g = grads[kind][i]
            errs.append((abs(g - fd) / max(abs(fd), abs(g)), kind, int(i), g, fd))
            taken += 1
            if taken == n:
                break
        assert taken == n, (kind, taken)
    errs.sort(reverse=True)
    assert len(errs) == 200
    assert errs[0][0] <= 1e-3, (errs[:5], kinked)


class RenderFn(torch.autograd.Function):
    """Test-harness autograd wrapper: forward renders, backward calls the
    library's adjoint with the upstream dL/drgb (visibility recomputed)."""

    @staticmethod
    def forward(ctx, positions, colors, texture, renderer, dscene, views):
        out = [torch.zeros(v.width * v.height * 3, device="cuda") for v in views]
        diff.forward(renderer, dscene, views, out, positions=positions.contiguous(), colors=colors.contiguous(),
                     texture=texture.contiguous())
        ctx.save_for_backward(positions, colors, texture)
        ctx.renderer, ctx.dscene, ctx.views = renderer, dscene, views
        return torch.stack(out)

    @staticmethod
    def backward(ctx, grad_out):
        positions, colors, texture = ctx.saved_tensors
        gp, gc, gt = torch.zeros_like(positions), torch.zeros_like(colors), torch.zeros_like(texture)
        grads = [grad_out[i].contiguous() for i in range(grad_out.shape[0])]
        diff.backward(ctx.renderer, ctx.dscene, ctx.views, gp, gc, gt, grad_rgb=grads,
                      positions=positions.contiguous(), colors=colors.contiguous(), texture=texture.contiguous())
        return gp, gc, gt, None, None, None


def test_autograd_wrapper_matches_and_descends(renderer, su):
    targets = torch.stack(su.render(renderer, su.target_scene))
    pos = su.scene.positions.clone().requires_grad_(True)
    col = su.scene.colors.clone().requires_grad_(True)
    tex = su.scene.texture.clone().requires_grad_(True)
    rgb = RenderFn.apply(pos, col, tex, renderer, su.scene, su.views)
    loss = ((rgb - targets) ** 2).sum() * su.scale
    loss.backward()
    su.render(renderer)
    l2, gp, gc, gt = gpu_grads(renderer, su, list(targets))
    assert abs(loss.item() - l2) <= 1e-4 * abs(l2)
    # the wrapper's upstream gradient is torch's 2 (rgb - target) scale, the
    # fused path forms it inside the kernel; both sum through fp32 atomics in
    # any order, and position gradients (long chains, cancellation near
    # vertices) differ by about 1e-4 relative between the two
    for a, b, tol in ((pos.grad, gp, 5e-4), (col.grad, gc, 1e-4), (tex.grad, gt, 1e-4)):
        a = a.cpu().numpy().reshape(-1)
        assert np.linalg.norm(a - b) <= tol * np.linalg.norm(b) + 1e-12
    # a few steps of gradient descent on colour and texture lower the loss
    losses = []
    with torch.no_grad():
        c, t = col.detach().clone(), tex.detach().clone()
    for _ in range(5):
        c.requires_grad_(True)
        t.requires_grad_(True)
        rgb = RenderFn.apply(pos.detach(), c, t, renderer, su.scene, su.views)
        loss = ((rgb - targets) ** 2).sum() * su.scale
        loss.backward()
        losses.append(loss.item())
        with torch.no_grad():
            c = (c - 2000.0 * c.grad).detach()
            t = (t - 2000.0 * t.grad).detach()
    assert losses[-1] < losses[0]


def test_captured_step_matches_eager(renderer, su):
    """Zero + forward + backward captured in one graph (visibility recomputed
    in the backward pass) gives the eager forward image exactly and the
    eager gradients to fp32-atomic reordering, on every replay."""
    targets = su.render(renderer, su.target_scene)
    ref_rgb = su.render(renderer)
    ref_loss, rp, rc, rt = gpu_grads(renderer, su, targets)
    rgb = [torch.empty(W * H * 3, device="cuda") for _ in su.views]
    gp = torch.full_like(su.scene.positions, 7.0)
    gc = torch.full_like(su.scene.colors, 7.0)
    gt = torch.full_like(su.scene.texture, 7.0)
    loss = torch.full((1,), 7.0, device="cuda")
    g = diff.capture_step(renderer, su.scene, su.views, rgb_out=rgb, targets=targets, grad_positions=gp,
                          grad_colors=gc, grad_texture=gt, scale=su.scale, loss=loss)
    try:
        assert g.kernel_count() >= 10
        for _ in range(2):
            for t in rgb:
                t.fill_(-1.0)
            g.launch()
            torch.cuda.synchronize()
            for a, b in zip(rgb, ref_rgb):
                assert torch.equal(a, b)
            assert abs(loss.item() - ref_loss) <= 1e-5 * abs(ref_loss)
            for a, b in ((gp, rp), (gc, rc), (gt, rt)):
                a = a.cpu().numpy().reshape(-1)
                assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b)
    finally:
        g.close()
    su._ids = None


def test_adjoint_graph_rejects_bad_passes(renderer, su):
    with pytest.raises(abi.VkgvError):
        diff.capture_step(renderer, su.scene, su.views, passes=8)
    with pytest.raises(abi.VkgvError):
        # backward without a target or an upstream gradient
        diff.capture_step(renderer, su.scene, su.views, passes=abi.DIFF_BACKWARD)


def test_uneven_views_forward_and_gradients(renderer):
    """Views of different sizes (partial 512-pixel chunks, a 33 x 17 and a
    512 x 40 view) in one call: the persistent shade maps every chunk to its
    view and pixels, for the forward image and the gradients."""
    sizes = [(96, 64), (200, 150), (33, 17), (512, 40)]
    rng = np.random.default_rng(9)
    mesh = scene.icosphere(3)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3)).astype(np.float32)
    texture = rng.uniform(0, 1, size=(64, 64, 3)).astype(np.float32)
    sc = diff.DiffScene.create(mesh, colors, texture)
    cams, views = [], []
    for w, h in sizes:
        v = rng.normal(size=3)
        eye = 3.0 * v / np.linalg.norm(v)
        cam = scene.camera(tuple(eye), (0, 0, 0), scene.safe_up(eye, (0, 0, 0)), 60.0, w / h)
        cams.append(cam)
        views.append(diff.DiffViewBuffers.allocate(w, h, cam))
    out = [torch.zeros(w * h * 3, device="cuda") for w, h in sizes]
    diff.forward(renderer, sc, views, out)
    torch.cuda.synchronize()
    ids = [v.ids() for v in views]
    assert all((i != abi.VISBUFFER_CLEAR).any() for i in ids)
    for (w, h), cam, o, idv in zip(sizes, cams, out, ids):
        _, ref, _ = ob.diff_f64(mesh, mesh.positions, colors, mesh.uvs, texture, vp_of(cam), w, h, idv, want_rgb=True)
        assert np.abs(o.cpu().numpy() - ref).max() < 5e-4
    targets = [rng.uniform(0, 1, size=w * h * 3).astype(np.float32) for w, h in sizes]
    scale = 1.0 / (3 * sum(w * h for w, h in sizes))
    gp, gc, gt = torch.zeros_like(sc.positions), torch.zeros_like(sc.colors), torch.zeros_like(sc.texture)
    loss = torch.zeros(1, device="cuda")
    diff.backward(renderer, sc, views, gp, gc, gt, targets=[torch.from_numpy(t).cuda() for t in targets],
                  scale=scale, loss=loss)
    torch.cuda.synchronize()
    ref_loss, ref = 0.0, None
    for (w, h), cam, t, idv in zip(sizes, cams, targets, ids):
        lv, _, g = ob.diff_f64(mesh, mesh.positions, colors, mesh.uvs, texture, vp_of(cam), w, h, idv, target=t,
                               scale=scale, want_grads=True)
        ref_loss += lv
        ref = g if ref is None else tuple(a + b for a, b in zip(ref, g))
    assert abs(float(loss.item()) - ref_loss) <= 1e-4 * abs(ref_loss)
    for name, g, r in (("positions", gp, ref[0]), ("colors", gc, ref[1]), ("texels", gt, ref[2])):
        g = g.cpu().numpy().reshape(-1)
        assert np.linalg.norm(g - r) / np.linalg.norm(r) < 1e-3, name
