"""Pins the CPU oracle to the reference (CPU only).

Fixtures in tests/golden/ were made by tests/golden/make_golden.py from the reference's own test
scenes (tests/test_single_gaussian.py, tests/test_multiple_gaussians.py) and from FP64
restatements of its SH recurrence and Adam rule.
"""
import math

import numpy as np
import pytest

FP16_ALPHA_BOUND = 2.0 ** -13 * 2.2  # half an fp16 ulp of alpha in [0.25, 0.5), times the colour sum bound


def _scene(golden, name):
    p = name + "_"
    return {k: golden[p + k] for k in ("mean", "log_scale", "color", "rotation", "logit_opacity", "bg",
                                       "alpha_threshold", "t_threshold")}


def _run_oracle(O, golden, name, bvh=False):
    s = _scene(golden, name)
    a_thr = float(s["alpha_threshold"])
    geom, l2w, aabb, vis = O.snapshot(s["mean"], s["rotation"], s["log_scale"], s["logit_opacity"][:, 0], a_thr)
    live = O.forward_prep(s["logit_opacity"][:, 0], a_thr)
    cfg = O.TraceConfig(alpha_threshold=a_thr, t_threshold=float(s["t_threshold"]), bg=tuple(s["bg"]))
    tree = O.Bvh(aabb, vis) if bvh else None
    out = O.trace_forward(golden["rays_o"], golden["rays_d"], geom, live, s["color"], vis, cfg, bvh=tree)
    return s, cfg, geom, l2w, out


NAMES = ["single_a0.01", "single_a0.3", "multi_t0.0", "multi_t0.5"]


@pytest.mark.parametrize("name", NAMES)
def test_oracle_image_matches_reference_rule(oracle, golden, name):
    """Against the reference CUDA rule evaluated in FP64 (fp16 keys, 32-slot passes, tail
    estimate): equal to float32 rounding except where an fp16 rounding midpoint separates the
    FP64 and FP32 alpha (rare pixels, bounded by half an fp16 ulp of alpha)."""
    s, cfg, *_ , out = _run_oracle(oracle, golden, name)
    diff = np.abs(out["rgb"] - golden[name + "_rule64_rgb"]).max(axis=1)
    assert np.mean(diff < 1e-6) >= 0.99
    assert diff.max() < FP16_ALPHA_BOUND


@pytest.mark.parametrize("name", NAMES)
def test_oracle_image_matches_reference_tests(oracle, golden, name):
    """Against the reference tests' FP64 loops: those composite with exact alpha, the reference
    kernel with fp16 alpha; the difference is bounded by the fp16 quantisation of alpha.  PSNR
    (peak 1) at least 60 dB (85-102 dB on these scenes)."""
    s, cfg, *_ , out = _run_oracle(oracle, golden, name)
    ref = golden[name + "_ref64_rgb"]
    err = np.abs(out["rgb"] - ref)
    assert err.mean() < 1e-4
    assert err.max() < 3e-4
    assert 10.0 * math.log10(1.0 / np.mean(err.astype(np.float64) ** 2)) >= 60.0


@pytest.mark.parametrize("name", NAMES)
def test_oracle_gradients_match_reference_tests(oracle, golden, name):
    """Gradients of the L1 loss against the reference tests' FP64 autograd, at the reference
    tests' own tolerance (abs 1e-4, tests/test_single_gaussian.py:228-232)."""
    s, cfg, geom, l2w, out = _run_oracle(oracle, golden, name)
    grad = oracle.trace_backward(32, 32, golden["rays_o"], golden["rays_d"], out, golden[name + "_ref64_grad_out"],
                                 geom, l2w, s["logit_opacity"], s["log_scale"], s["rotation"], s["color"], cfg)
    pairs = [(slice(0, 4), "rotation"), (slice(4, 7), "mean"), (slice(7, 8), "logit_opacity"),
             (slice(8, 11), "log_scale"), (slice(12, 15), "color")]
    for sl, key in pairs:
        ref = golden[name + "_ref64_grad_" + key]
        assert np.abs(grad[:, sl] - ref).max() < 1e-4, key


@pytest.mark.parametrize("name", NAMES)
def test_oracle_bvh_traversal_equals_brute_force(oracle, golden, name):
    *_, a = _run_oracle(oracle, golden, name)
    *_, b = _run_oracle(oracle, golden, name, bvh=True)
    assert np.array_equal(a["nhit"], b["nhit"])
    assert np.array_equal(a["nacc"], b["nacc"])
    assert np.array_equal(a["ids"], b["ids"])
    assert np.array_equal(a["T"], b["T"])
    assert np.array_equal(a["rem"], b["rem"])


@pytest.mark.parametrize("deg", [0, 1, 2, 3])
def test_oracle_sh_matches_reference_recurrence(oracle, golden_sh, deg):
    g = golden_sh
    col = oracle.sh_forward(deg, g["mean"], g["cam"], g["dc"][:, 0, :], g["rest"])
    assert np.abs(col - g[f"deg{deg}_colour"]).max() < 5e-7
    vis = np.ones(col.shape[0], np.uint8)
    gdc, grest, gm = oracle.sh_backward(deg, g["mean"], g["cam"], g["rest"], col, g[f"deg{deg}_grad_colour"], vis,
                                        np.zeros((col.shape[0], 3), np.float32))
    assert np.abs(gdc - g[f"deg{deg}_grad_dc"][:, 0, :]).max() < 1e-6
    assert np.abs(grest - g[f"deg{deg}_grad_rest"]).max() < 2e-6
    assert np.abs(gm - g[f"deg{deg}_grad_mean"]).max() < 2e-6


@pytest.mark.parametrize("step", [1, 7, 1000])
def test_oracle_adam_matches_fp64_rule(oracle, golden_sh, step):
    """cuda/opt/adam.cu:13-22 (bias-correction exponent step + 1) against its FP64 restatement."""
    g = golden_sh
    n = 16  # the 64 golden values ride in the rotation group ([16, 4])
    st = {}
    for name, width in (("channels", 3), ("opacity", 1), ("mean", 3), ("rotation", 4), ("scale", 3), ("sh_dc", 3),
                        ("sh_rest", 0)):
        for pre in ("", "g_", "m_", "v_"):
            st[pre + name] = np.zeros(n * width, np.float32)
    st["rotation"], st["m_rotation"], st["v_rotation"], st["g_rotation"] = (
        g["adam_in_" + k].copy() for k in ("p", "m", "v", "g"))
    oracle.adam_step(st, {"rotation": 0.01}, n, 0, step, zero_grads=True)
    assert np.allclose(st["rotation"], g[f"adam_step{step}_p"], rtol=1e-6, atol=1e-7)
    assert np.allclose(st["m_rotation"], g[f"adam_step{step}_m"], rtol=1e-6, atol=1e-9)
    assert np.allclose(st["v_rotation"], g[f"adam_step{step}_v"], rtol=1e-6, atol=1e-12)
    assert not st["g_rotation"].any()


def _ulp_err(got, ref):
    got = np.float32(got)
    ref32 = np.float32(ref)
    if not np.isfinite(ref32):
        return 0 if got == ref32 else 99
    return abs(float(got) - ref) / float(np.spacing(np.abs(ref32)))


def test_own_exp_log_accuracy(oracle):
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(-103, 88, 3000), rng.uniform(-1, 1, 2000), rng.uniform(-20, 0, 2000)])
    worst = max(_ulp_err(oracle.expf(float(np.float32(x))), math.exp(float(np.float32(x)))) for x in xs)
    assert worst <= 2.0
    ys = np.concatenate([np.exp(rng.uniform(-80, 80, 3000)), rng.uniform(0.5, 2, 2000), rng.uniform(1e-3, 1e3, 2000)])
    worst = max(_ulp_err(oracle.logf(float(np.float32(y))), math.log(float(np.float32(y)))) for y in ys)
    assert worst <= 2.5
    assert oracle.expf(0.0) == 1.0
    assert oracle.logf(1.0) == 0.0


def test_half_rounding_matches_ieee(oracle):
    rng = np.random.default_rng(1)
    v = np.concatenate([rng.uniform(0, 70000, 4000), np.exp(rng.uniform(-20, 11, 4000)), [0.0, 2.0 ** -25,
                        2.0 ** -24, 65504.0, 65520.0, 1e-8]]).astype(np.float32)
    lib = oracle.lib()
    for x in v:
        h = lib.orc_f2h(float(x))
        assert h == int(np.float16(x).view(np.uint16)), x
        assert lib.orc_h2f(h) == float(np.float16(x))


def test_maxalpha_product_is_correctly_rounded(oracle):
    rng = np.random.default_rng(2)
    lib = oracle.lib()
    bad = 0
    for _ in range(5000):
        a, b = np.float32(rng.uniform(0, 1)), np.float32(rng.uniform(0, 1))
        ref = np.float32(0.9999 * float(a) * float(b))
        bad += lib.orc_maxalpha_mul(float(a), float(b)) != ref
    assert bad <= 2


def test_lbvh_nodes_hold_their_leaf_counts(oracle):
    """Node words 14 and 15 of the LBVH (the forward's frontier walk reads them instead of loading
    the children): the leaves below the node and below its first child, consistent through the
    whole tree and with every leaf below the root exactly once."""
    from gray_gb300 import synthetic

    sc = synthetic.clustered_scene(5000, seed=11)
    _, _, aabb, vis = oracle.snapshot(sc.mean, sc.rotation, sc.scale, sc.opacity[:, 0])
    tree = oracle.Bvh(aabb, vis)
    nodes = tree.nodes
    links = nodes[:, 12:14].copy().view(np.uint32)
    counts = nodes[:, 14:16].copy().view(np.uint32)
    leaf_bit = np.uint32(0x80000000)

    def leaves(child):
        return 1 if child & leaf_bit else int(counts[child, 0])

    seen = []
    stack = [0]
    while stack:
        i = stack.pop()
        c0, c1 = int(links[i, 0]), int(links[i, 1])
        assert counts[i, 1] == leaves(c0), i
        assert counts[i, 0] == leaves(c0) + leaves(c1), i
        for c in (c0, c1):
            if c & leaf_bit:
                seen.append(c & ~leaf_bit)
            else:
                stack.append(c)
    assert counts[0, 0] == sc.n
    assert sorted(seen) == list(range(sc.n))


def _random_tree(oracle, n, seed):
    rng = np.random.default_rng(seed)
    mean = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    rot = rng.standard_normal((n, 4)).astype(np.float32)
    scale = rng.normal(-3, 0.3, (n, 3)).astype(np.float32)
    opac = rng.standard_normal(n).astype(np.float32)
    _, _, aabb, vis = oracle.snapshot(mean, rot, scale, opac)
    return oracle.Bvh(aabb, vis), aabb, rng


def test_refit_climb_equals_top_down_refit(oracle):
    """The GPU refit's bottom-up protocol (visit counters, second arriver climbs on) gives the
    top-down refit's node and root boxes, with no status bit, on trees of several sizes."""
    for n in (1, 2, 3, 257, 1000):
        tree, aabb, rng = _random_tree(oracle, n, n)
        aabb2 = aabb.copy()
        aabb2[:, :3] -= rng.uniform(0, 0.1, (n, 3)).astype(np.float32)
        tree.refit(aabb2)
        nodes, root = tree.nodes, tree.root_box
        tree.refit(aabb)
        assert tree.refit_climb(aabb2) == 0
        assert np.array_equal(tree.nodes, nodes)
        assert np.array_equal(tree.root_box, root)


def test_refit_climb_reports_a_corrupt_parent_chain(oracle):
    """A parent link that points back down the tree makes a cycle: the climb stops after 128 levels
    and reports GRAY_STATUS_REFIT_TIMEOUT (bit 4) instead of looping (the mistake is planted in the
    oracle's copy of the tree, on the CPU)."""
    tree, aabb, _ = _random_tree(oracle, 1000, 7)
    nodes = tree.nodes
    links = nodes[:, 12:14].view(np.uint32)
    internal = links[0][links[0] < 0x80000000]
    assert internal.size > 0
    child = int(internal[0])
    tree.int_parent[0] = child  # the root's parent is now its own child
    assert tree.refit_climb(aabb) & 4 == 4


def _lines(rng, n, dist, lo_mag, ld_mag):
    """Object-space rays (lo, ld) whose lines pass at distance `dist` from the centre."""
    e = rng.standard_normal((n, 3))
    e /= np.linalg.norm(e, axis=1, keepdims=True)
    w = rng.standard_normal((n, 3))
    w -= np.sum(w * e, axis=1, keepdims=True) * e
    w /= np.linalg.norm(w, axis=1, keepdims=True)
    along = np.sqrt(np.maximum(lo_mag ** 2 - dist ** 2, 0.0))[:, None]
    lo = w * dist[:, None] - along * e
    ld = e * ld_mag[:, None]
    return lo.astype(np.float32), ld.astype(np.float32)


def test_hit_pretest_never_drops_a_hit(oracle):
    """The kernels' division-free pretest (cross product with a rounding margin) keeps every pair
    the exact hit decision accepts: lines within 1e-3 and 1e-6 of the unit sphere's surface,
    object-space origins from 1e-3 to 1e11 away, direction lengths from 1e-15 to 1e15, zero
    components, infinities and NaNs.  At the benchmark's magnitudes it keeps almost nothing else."""
    rng = np.random.default_rng(7)
    n = 400_000
    for spread, lo_exp, ld_exp in ((1e-3, (-3, 4), (-15, 15)), (1e-6, (-3, 4), (-1, 3)),
                                   (1e-3, (4, 11), (-3, 3)), (3.0, (-3, 11), (-15, 15))):
        dist = 1.0 + (rng.random(n) - 0.5) * 2 * spread if spread < 1 else rng.random(n) * spread
        lo, ld = _lines(rng, n, dist, 10.0 ** rng.uniform(*lo_exp, n), 10.0 ** rng.uniform(*ld_exp, n))
        ld[::13, 1] = 0.0
        lo[::17, 2] = 0.0
        accepted, kept, dropped = oracle.pretest_check(lo, ld)
        assert dropped == 0, (spread, lo_exp, ld_exp)
        assert accepted > n // 20
    special = np.array([np.inf, -np.inf, np.nan, 1e-40, 0.0, 3e38], dtype=np.float32)
    lo, ld = _lines(rng, 6 * 6 * 3, np.ones(108), np.full(108, 5.0), np.ones(108))
    for i in range(108):
        (lo if i % 2 else ld)[i, i % 3] = special[(i // 3) % 6]
    assert oracle.pretest_check(lo, ld)[2] == 0
    # magnitudes of the benchmark scene: |lo| 10-2000, |ld| 1-1000
    dist = rng.random(n) * 2.0
    lo, ld = _lines(rng, n, dist, 10.0 ** rng.uniform(1, 3.3, n), 10.0 ** rng.uniform(0, 3, n))
    accepted, kept, dropped = oracle.pretest_check(lo, ld)
    assert dropped == 0 and kept - accepted <= max(2, accepted // 1000)


def test_ellipsoid_cull_never_culls_a_reachable_ellipsoid(oracle):
    """The kernels' ellipsoid-plane cull (squared extent against the squared gap, 6e-5 margin, gaps
    below 2^-60 never culled), given the frustum plane's threshold with its rounding margin
    (1e-5 |n|_1 (3m + |o|_1), m bounding the coordinates), culls only ellipsoids that FP64 puts
    entirely below the plane: planes within 1e-4 (relative) of the ellipsoid's top on both sides,
    extents from 1e-25 to 1e15, scenes of 1e-20 (subnormal squares), scaled normals, and degenerate
    (flat) ellipsoids."""
    rng = np.random.default_rng(3)
    n = 300_000
    for ext_exp, mu_exp, near in (((-3, 1), (-3, 3), 1e-4), ((-25, -15), (-3, 3), 1e-4), ((5, 15), (-3, 3), 1e-4),
                                  ((-25, 15), (-3, 3), 0.5), ((-25, -20), (-24, -20), 1e-4)):
        q = rng.standard_normal((n, 4))
        q /= np.linalg.norm(q, axis=1, keepdims=True)
        w_, x, y, z = q.T
        R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w_ * z), 2 * (x * z + w_ * y)], -1),
                      np.stack([2 * (x * y + w_ * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w_ * x)], -1),
                      np.stack([2 * (x * z - w_ * y), 2 * (y * z + w_ * x), 1 - 2 * (x * x + y * y)], -1)], 1)
        s = 10.0 ** rng.uniform(*ext_exp, (n, 3))
        s[::7, 2] = 0.0                                   # flat ellipsoids
        L = R * s[:, None, :]
        mu = rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(*mu_exp, (n, 1))
        nrm = rng.standard_normal((n, 3)) * 10.0 ** rng.uniform(-2, 2, (n, 1))
        l2w = np.concatenate([L, mu[:, :, None]], axis=2).reshape(n, 12).astype(np.float32)
        L32, mu32, n32 = l2w.reshape(n, 3, 4)[:, :, :3].astype(np.float64), l2w.reshape(n, 3, 4)[:, :, 3].astype(
            np.float64), nrm.astype(np.float32).astype(np.float64)
        top = np.sum(n32 * mu32, axis=1) + np.linalg.norm(np.einsum("nrc,nr->nc", L32, n32), axis=1)
        scale = np.abs(top) + np.linalg.norm(np.einsum("nrc,nr->nc", L32, n32), axis=1)
        plane = top + rng.uniform(-near, near, n) * scale
        m = np.max(np.abs(mu32), axis=1) + np.max(np.abs(L32), axis=(1, 2)) * 3.0
        mell = 1e-5 * np.sum(np.abs(n32), axis=1) * 3.0 * m + 1e-30
        thr = (plane.astype(np.float32) - mell.astype(np.float32)).astype(np.float32)
        culled, wrong = oracle.cull_check(nrm, l2w, thr, plane)
        assert wrong == 0, (ext_exp, mu_exp, near, culled, wrong)
        assert culled > n // 50 or mu_exp[1] < -15  # (tiny scenes: gaps below 2^-60 are never culled)
