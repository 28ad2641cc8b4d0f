"""CPU check of the float64 adjoint reference: its analytic gradient against
central finite differences of its own loss at fixed visibility (ids from the
oracle raster).  This pins the derivation that the GPU kernel also follows."""
import numpy as np

from oracle import binding as ob
from vk_gltf_viewer_gb300 import scene


def test_f64_gradient_matches_finite_differences(built):
    rng = np.random.default_rng(9)
    mesh = scene.icosphere(2)
    nv = mesh.positions.shape[0]
    colors = rng.uniform(0, 1, size=(nv, 3))
    tex = rng.uniform(0, 1, size=(32, 32, 3))
    host = scene.HostScene(meshes=[mesh], prim_materials=[1],
                           materials=np.concatenate([scene.default_material(), scene.make_material()]),
                           transforms=scene.to_column_major(np.eye(4))[None, :].copy(), node_meshes=[[0]])
    osc = ob.OracleScene(host)
    w = h = 48
    cams = [scene.camera((0.3, 0.4, 2.8), (0, 0, 0), (0, 1, 0), 60.0, 1.0),
            scene.camera((-2.5, 1.0, -1.0), (0, 0, 0), (0, 1, 0), 60.0, 1.0)]
    ids = [ob.frame(osc, c, w, h, 0)["ids"] for c in cams]
    targets = [rng.uniform(0, 1, size=w * h * 3).astype(np.float32) for _ in cams]
    vps = [np.frombuffer(bytes(c), np.float32)[32:48].copy() for c in cams]
    kw = dict(uv_scale=(2.0, 1.5), uv_offset=(0.1, -0.2), uv_rotation=0.3, albedo=(0.9, 0.8, 1.0))

    def loss_and_grads(pos, col, tx, grads=True):
        total, g = 0.0, None
        for vp, i, t in zip(vps, ids, targets):
            l, _, gg = ob.diff_f64(mesh, pos, col, mesh.uvs, tx, vp, w, h, i, target=t, scale=1e-3,
                                   want_grads=grads, **kw)
            total += l
            if grads:
                g = gg if g is None else tuple(a + b for a, b in zip(g, gg))
        return total, g

    base = {"pos": mesh.positions.astype(np.float64), "col": colors, "tex": tex}
    _, (gp, gc, gt) = loss_and_grads(base["pos"], base["col"], base["tex"])
    grads = {"pos": gp, "col": gc, "tex": gt}
    # the loss is quadratic in colours and texels (central differences are
    # exact for any step) and smooth in positions at fixed visibility
    steps = {"pos": 1e-6, "col": 1e-3, "tex": 1e-3}
    for kind, n in (("pos", 20), ("col", 20), ("tex", 20)):
        h_fd = steps[kind]
        nz = np.nonzero(np.abs(grads[kind]) > 1e-9)[0]
        for i in rng.choice(nz, size=n, replace=False):
            vals = []
            for sgn in (1.0, -1.0):
                arrs = {k: v.copy() for k, v in base.items()}
                arrs[kind].reshape(-1)[i] += sgn * h_fd
                vals.append(loss_and_grads(arrs["pos"], arrs["col"], arrs["tex"], grads=False)[0])
            fd = (vals[0] - vals[1]) / (2 * h_fd)
            g = grads[kind][i]
            assert abs(g - fd) <= 1e-5 * max(abs(fd), abs(g)) + 1e-12, (kind, i, g, fd)
