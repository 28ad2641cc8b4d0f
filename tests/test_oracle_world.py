"""The oracle's world update (world.cpp:187-345, assets.hpp:51-113) on CPU:
its series and slerp against float64 math, the sampler's boundary, looping
and interpolation rules against a float32 restatement, T * R * S against
float64 matrices, and the depth-first transform and draw numbering on hand
trees (nodes without meshes, a node reached twice, several and empty
primitives, a path deeper than 64)."""
import math

import numpy as np
import pytest

from oracle import binding as ob
from vk_gltf_viewer_gb300 import abi
from vk_gltf_viewer_gb300.world import HostWorld, Sampler, make_nodes, quat_axis_angle

f32 = np.float32


def test_series_match_libm():
    """Both float series stay within 2.5e-7 relative of the float64 functions."""
    for x in np.linspace(1e-6, math.pi / 2, 2049).astype(np.float32):
        assert abs(ob.sin_series(float(x)) - math.sin(x)) <= 2.5e-7 * math.sin(x)
    for z in np.linspace(1e-6, math.sin(math.pi / 8), 2049).astype(np.float32):
        assert abs(ob.asin_series(float(z)) - math.asin(z)) <= 2.5e-7 * math.asin(z)


def _slerp64(a, b, t):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    d = float(a @ b)
    if d < 0:
        b, d = -b, -d
    th = math.acos(min(1.0, d))
    if th < 1e-6:
        return (1 - t) * a + t * b
    return (math.sin((1 - t) * th) * a + math.sin(t * th) * b) / math.sin(th)


def test_slerp_matches_float64():
    rng = np.random.default_rng(3)
    worst = 0.0
    for _ in range(2000):
        a = rng.normal(size=4)
        a /= np.linalg.norm(a)
        b = rng.normal(size=4)
        b /= np.linalg.norm(b)
        if rng.random() < 0.2:  # nearly equal keys
            b = a + rng.normal(scale=1e-7, size=4)
            b /= np.linalg.norm(b)
        a32, b32 = a.astype(f32), b.astype(f32)
        t = float(rng.random())
        got = ob.slerp(a32, b32, t)
        exp = _slerp64(a32, b32, f32(t))
        worst = max(worst, float(np.abs(got - exp).max()))
    assert worst < 1e-6, worst
    # the shorter arc: a key and its negation interpolate to the key
    q = quat_axis_angle((0, 1, 0), 0.3)
    assert np.allclose(ob.slerp(q, -q, 0.5), q, atol=1e-7)


def _sample32(times, vals, interp, time, rotation=False):
    """Float32 restatement of AnimationSampler::sample with the pinned order."""
    times = times.astype(f32)
    tt = f32(math.fmod(f32(time), times[-1]))
    i = int(np.searchsorted(times, tt, side="left"))
    cubic = interp == abi.INTERP_CUBICSPLINE
    if i == 0:
        return vals[1 if cubic else 0]
    if i == len(times):
        return vals[-2 if cubic else -1]
    t = (tt - times[i - 1]) / (times[i] - times[i - 1])
    if interp == abi.INTERP_STEP:
        return vals[i - 1]
    if interp == abi.INTERP_LINEAR:
        if rotation:
            return _slerp64(vals[i - 1], vals[i], t)
        return (f32(1) - t) * vals[i - 1] + t * vals[i]
    t2 = t * t
    t3 = t2 * t
    dt = times[i] - times[i - 1]
    h00 = (f32(2) * t3 - f32(3) * t2) + f32(1)
    h10 = (t3 - f32(2) * t2) + t
    h01 = f32(-2) * t3 + f32(3) * t2
    h11 = t3 - t2
    p0, m0, p1, m1 = vals[3 * (i - 1) + 1], vals[3 * (i - 1) + 2], vals[3 * i + 1], vals[3 * i]
    v = ((p0 * h00 + (m0 * h10) * dt) + p1 * h01) + (m1 * h11) * dt
    if rotation:
        v = v / np.sqrt(((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]) + v[3] * v[3])
    return v


@pytest.mark.parametrize("interp", [abi.INTERP_STEP, abi.INTERP_LINEAR, abi.INTERP_CUBICSPLINE])
def test_sampler_rules(interp):
    rng = np.random.default_rng(interp)
    times = np.array([0.25, 0.5, 1.25, 2.0], f32)
    n = times.size * (3 if interp == abi.INTERP_CUBICSPLINE else 1)
    vals = rng.normal(size=(n, 3)).astype(f32)
    # before the first key, on every key, between keys, past the end (looped),
    # negative time, and exactly the last key (fmod gives 0)
    probe = [0.0, 0.1, 0.25, 0.3, 0.5, 0.9, 1.25, 1.7, 2.0, 2.6, 4.3, -0.4, 0.2500001]
    for t in probe:
        got = ob.anim_sample(times, vals, interp, t, abi.PATH_TRANSLATION)
        exp = _sample32(times, vals, interp, t)
        assert np.array_equal(got, np.asarray(exp, f32)), (t, got, exp)


def test_rotation_sampler_rules():
    times = np.array([0.0, 1.0, 3.0], f32)
    keys = np.stack([quat_axis_angle((0, 0, 1), a) for a in (0.0, 1.0, 2.5)])
    for t in (0.0, 0.4, 1.0, 2.2, 3.7):
        got = ob.anim_sample(times, keys, abi.INTERP_LINEAR, t, abi.PATH_ROTATION)
        assert np.abs(got - _sample32(times, keys, abi.INTERP_LINEAR, t, True)).max() < 1e-6
    tang = np.random.default_rng(1).normal(scale=0.1, size=(3, 2, 4)).astype(f32)
    cub = np.concatenate([tang[:, :1], keys[:, None], tang[:, 1:]], 1).reshape(9, 4)
    for t in (0.0, 0.4, 1.0, 2.2, 3.7):
        got = ob.anim_sample(times, cub, abi.INTERP_CUBICSPLINE, t, abi.PATH_ROTATION)
        exp = np.asarray(_sample32(times, cub, abi.INTERP_CUBICSPLINE, t, True), f32)
        assert np.array_equal(got, exp), (t, got, exp)


def _mat64(t, q, s):
    x, y, z, w = (float(v) for v in q)
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
                  [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
                  [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)]])
    M = np.eye(4)
    M[:3, :3] = R * np.asarray(s, np.float64)[None, :]
    M[:3, 3] = t
    return M


def test_trs_matrix_matches_float64():
    rng = np.random.default_rng(9)
    for _ in range(200):
        t = rng.normal(size=3).astype(f32)
        q = quat_axis_angle(rng.normal(size=3), rng.uniform(0, 6.3))
        s = rng.uniform(0.2, 3, 3).astype(f32)
        got = ob.trs_matrix(t, q, s).reshape(4, 4).T
        assert np.allclose(got, _mat64(t, q, s), rtol=0, atol=3e-6)


def hand_world():
    """root(0) -> a(1, mesh 0) -> b(2, no mesh) -> c(3, mesh 1)
                -> d(4, mesh 2), and root 5 (mesh 0) whose child is b (a node
    reached twice).  mesh 0 = primitives [0, 1], mesh 1 = [2], mesh 2 = [1, 3]
    (primitive 3 has no meshlets)."""
    nodes = make_nodes(6)
    kids = [1, 4, 2, 3, 2]
    nodes[0]["first_child"], nodes[0]["child_count"] = 0, 2
    nodes[1]["first_child"], nodes[1]["child_count"] = 2, 1
    nodes[2]["first_child"], nodes[2]["child_count"] = 3, 1
    nodes[5]["first_child"], nodes[5]["child_count"] = 4, 1
    nodes[1]["mesh_index"], nodes[3]["mesh_index"], nodes[4]["mesh_index"], nodes[5]["mesh_index"] = 0, 1, 2, 0
    rng = np.random.default_rng(4)
    for n in range(6):
        nodes[n]["translation"] = rng.normal(size=3)
        nodes[n]["rotation"] = quat_axis_angle(rng.normal(size=3), rng.uniform(0, 3))
        nodes[n]["scale"] = rng.uniform(0.5, 2.0, 3)
    samplers = [Sampler(np.array([0.0, 1.0], f32), np.array([[0, 0, 0], [1, 2, 3]], f32), abi.INTERP_LINEAR),
                Sampler(np.array([0.0, 2.0], f32),
                        np.stack([quat_axis_angle((1, 0, 0), 0.0), quat_axis_angle((1, 0, 0), 1.5)]),
                        abi.INTERP_LINEAR),
                Sampler(np.array([0.0, 0.5, 1.0], f32), np.array([[1, 1, 1], [2, 2, 2], [3, 3, 3]], f32),
                        abi.INTERP_STEP)]
    # two channels on node 2's translation: the later one wins
    channels = [(0, 2, abi.PATH_TRANSLATION, 0), (1, 1, abi.PATH_ROTATION, 0), (2, 4, abi.PATH_SCALE, 0),
                (2, 2, abi.PATH_TRANSLATION, 0), (0, 3, abi.PATH_WEIGHTS, 0)]
    return HostWorld(nodes=nodes, children=np.array(kids, np.uint32), roots=np.array([0, 5], np.uint32),
                     mesh_primitives=[[0, 1], [2], [1, 3]], primitive_meshlet_counts=np.array([3, 2, 4, 0], np.uint32),
                     samplers=samplers, channels=np.array(channels, np.uint32))


def test_hand_tree_draw_order():
    w = hand_world()
    d = ob.world_draws(w)
    # slots: a=0 (mesh 0), c=1 (mesh 1), d=2 (mesh 2), root5=3 (mesh 0), c again=4 (mesh 1)
    exp = []
    for slot, mesh in enumerate([0, 1, 2, 0, 1]):
        for p in w.mesh_primitives[mesh]:
            exp += [(p, m, slot) for m in range(int(w.primitive_meshlet_counts[p]))]
    assert np.array_equal(d, np.array(exp, np.uint32))
    assert w.meshlet_draw_count == len(exp)


def test_hand_tree_transforms():
    w = hand_world()
    for time in (0.0, 0.3, 0.75, 1.6):
        got = ob.world_transforms(w, time)
        assert got.shape == (5, 16)
        trs = {}
        for n in range(6):
            node = w.nodes[n]
            trs[n] = [node["translation"].astype(f32), node["rotation"].astype(f32), node["scale"].astype(f32)]
        # the animated values (the last channel on a path wins)
        tt = f32(time)
        trs[2][0] = np.asarray(_sample32(np.array([0.0, 0.5, 1.0], f32),
                                         np.array([[1, 1, 1], [2, 2, 2], [3, 3, 3]], f32), abi.INTERP_STEP, tt), f32)
        trs[1][1] = np.asarray(_sample32(np.array([0.0, 2.0], f32), w.samplers[1].output, abi.INTERP_LINEAR, tt,
                                         True), f32)
        trs[4][2] = trs[2][0]
        M = {n: _mat64(*trs[n]) for n in range(6)}
        chains = [[0, 1], [0, 1, 2, 3], [0, 4], [5], [5, 2, 3]]
        for slot, chain in enumerate(chains):
            exp = np.eye(4)
            for n in chain:
                exp = exp @ M[n]
            assert np.allclose(got[slot].reshape(4, 4).T, exp, rtol=1e-5, atol=2e-5), (time, slot)


def test_depth_limit():
    nodes = make_nodes(70)
    for n in range(69):
        nodes[n]["first_child"], nodes[n]["child_count"] = n, 1
    nodes["mesh_index"][69] = 0
    deep = HostWorld(nodes=nodes, children=np.arange(1, 70, dtype=np.uint32), roots=np.array([0], np.uint32),
                     mesh_primitives=[[0]], primitive_meshlet_counts=np.array([1], np.uint32))
    with pytest.raises(ValueError):
        ob.world_transforms(deep, 0.0)
    shallow = HostWorld(nodes=nodes[:64].copy(), children=np.arange(1, 64, dtype=np.uint32),
                        roots=np.array([0], np.uint32), mesh_primitives=[[0]],
                        primitive_meshlet_counts=np.array([1], np.uint32))
    shallow.nodes[63]["child_count"] = 0
    shallow.nodes[63]["mesh_index"] = 0
    assert ob.world_transforms(shallow, 0.0).shape == (1, 16)
