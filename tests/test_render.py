"""Headless ray march of the density (the viewer's volume shader,
SampleSmokeGUI/raycastingshader.h:10-70, as zqs_render_density / zqs_grid_render).

CPU: the oracle against a pure-Python float32 restatement of the shader text on
a few pixels, the viewer's default camera, and exact scaling properties.
GPU: the kernel against the oracle (RGB bit-identical; alpha = exp(-v) within
1e-6 relative, as CUDA's and the C library's expf may differ in the last
bits), the grid entry point on a simulated density, full-size properties and
argument checks.
"""
import math

import numpy as np
import pytest

from zq_smokesimulation_gb300 import capi
from zq_smokesimulation_gb300 import workloads as wl

f32 = np.float32
ALPHA_RTOL = 1e-6


def blob_density(W, H, D, seed=3):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(D), np.arange(H), np.arange(W), indexing="ij")
    c = np.array([0.45 * W, 0.4 * H, 0.55 * D])
    r2 = ((x - c[0]) / W) ** 2 + ((y - c[1]) / H) ** 2 + ((z - c[2]) / D) ** 2
    rho = np.exp(-r2 / 0.05) + 0.2 * rng.random((D, H, W))
    return np.ascontiguousarray(rho, np.float32)


def rotation(axis, angle):
    a = np.asarray(axis, np.float64)
    a = a / np.linalg.norm(a)
    K = np.array([[0, -a[2], a[1]], [a[2], 0, -a[0]], [-a[1], a[0], 0]])
    return np.eye(3) + math.sin(angle) * K + (1 - math.cos(angle)) * K @ K


def orbit_camera(img_w, img_h, W, H, D, axis=(0.3, 1.0, 0.2), angle=0.7, steps=64, scale=1.5):
    cam = capi.default_camera(img_w, img_h, W, H, D)
    R = rotation(axis, angle).astype(np.float32)
    cam.inv_view[:] = [float(v) for v in R.ravel()]
    eye = R.astype(np.float64) @ np.array([0.0, 0.0, 2.0])
    cam.eye[:] = [float(v) for v in eye.astype(np.float32)]
    cam.steps = steps
    cam.density_scale = scale
    return cam


def shader_pixel(vol, cam, px, py):
    """The fragment shader for one pixel in float32 scalar arithmetic."""
    D, H, W = vol.shape

    def at(i, j, k):
        if 0 <= i < W and 0 <= j < H and 0 <= k < D:
            return vol[k, j, i]
        return f32(0)

    def lerp(a, b, t):
        return f32(a + f32(t * f32(b - a)))

    def tex(s, t, r):
        s, t, r = (min(max(v, f32(0)), f32(1)) for v in (s, t, r))
        fx, fy, fz = f32(f32(s * f32(W)) - f32(0.5)), f32(f32(t * f32(H)) - f32(0.5)), f32(f32(r * f32(D)) - f32(0.5))
        x0, y0, z0 = np.floor(fx), np.floor(fy), np.floor(fz)
        ax, ay, az = f32(fx - x0), f32(fy - y0), f32(fz - z0)
        i, j, k = int(x0), int(y0), int(z0)
        e00, e10 = lerp(at(i, j, k), at(i + 1, j, k), ax), lerp(at(i, j + 1, k), at(i + 1, j + 1, k), ax)
        e01, e11 = lerp(at(i, j, k + 1), at(i + 1, j, k + 1), ax), lerp(at(i, j + 1, k + 1), at(i + 1, j + 1, k + 1), ax)
        return lerp(lerp(e00, e10, ay), lerp(e01, e11, ay), az)

    hw, hh = f32(f32(f32(cam.width) - f32(1)) / f32(2)), f32(f32(f32(cam.height) - f32(1)) / f32(2))
    d = [f32(f32(f32(px) + f32(0.5)) - hw), f32(f32(f32(py) + f32(0.5)) - hh), f32(-cam.focal)]
    ln = np.sqrt(f32(f32(f32(d[0] * d[0]) + f32(d[1] * d[1])) + f32(d[2] * d[2])))
    d = [f32(v / ln) for v in d]
    m = [f32(v) for v in cam.inv_view]
    r = [f32(f32(f32(m[3 * q] * d[0]) + f32(m[3 * q + 1] * d[1])) + f32(m[3 * q + 2] * d[2])) for q in range(3)]
    ln = np.sqrt(f32(f32(f32(r[0] * r[0]) + f32(r[1] * r[1])) + f32(r[2] * r[2])))
    r = [f32(v / ln) for v in r]
    eye, bmin, bmax, bsz = ([f32(v) for v in a] for a in (cam.eye, cam.box_min, cam.box_max, cam.box_size))
    with np.errstate(divide="ignore"):
        inv = [f32(f32(1) / v) for v in r]
    tb = [f32(inv[q] * f32(bmin[q] - eye[q])) for q in range(3)]
    tt = [f32(inv[q] * f32(bmax[q] - eye[q])) for q in range(3)]
    tmin = [np.fmin(tt[q], tb[q]) for q in range(3)]
    tmax = [np.fmax(tt[q], tb[q]) for q in range(3)]
    tnear = np.fmax(np.fmax(tmin[0], tmin[1]), np.fmax(tmin[0], tmin[2]))
    tfar = np.fmin(np.fmin(tmax[0], tmax[1]), np.fmin(tmax[0], tmax[2]))
    if not tfar > tnear:
        return np.array([0, 0, 0, 1], np.float32)
    pos = [f32(f32(f32(eye[q] + f32(r[q] * tnear)) - bmin[q]) / bsz[q]) for q in range(3)]
    steplen = f32(f32(tfar - tnear) / f32(cam.steps))
    step = [f32(f32(steplen * r[q]) / bsz[q]) for q in range(3)]
    steplen = f32(steplen / bsz[0])
    acc = f32(0)
    for _ in range(cam.steps):
        acc = f32(acc + f32(steplen * tex(*pos)))
        pos = [f32(pos[q] + step[q]) for q in range(3)]
    v = f32(acc * f32(cam.density_scale))
    return np.array([v, v, v, np.exp(-v)], np.float32)


def assert_image_equal(img, ref):
    np.testing.assert_array_equal(img[..., :3], ref[..., :3])
    np.testing.assert_allclose(img[..., 3], ref[..., 3], rtol=ALPHA_RTOL, atol=0)


def test_default_camera_is_the_viewers(zqs_lib):
    cam = capi.default_camera(1024, 768, 256, 128, 64)
    assert (cam.width, cam.height, cam.steps) == (1024, 768, 300) and cam.density_scale == 1.0
    assert cam.focal == f32(768 / 2.0 / math.atan(float(f32(40.0) / f32(360.0)) * math.pi))
    assert list(cam.eye) == [0.0, 0.0, 2.0] and list(cam.inv_view) == [1, 0, 0, 0, 1, 0, 0, 0, 1]
    xl, zl = f32(256) / f32(128), f32(64) / f32(128)
    assert list(cam.box_size) == [xl, 1.0, zl]
    assert list(cam.box_min) == [f32(-0.5 * xl), -0.5, f32(-0.5 * zl)] and list(cam.box_max) == [f32(0.5 * xl), 0.5, f32(0.5 * zl)]


@pytest.mark.parametrize("orbit", [False, True])
def test_oracle_matches_shader_restatement(oracle32, orbit):
    W, H, D = 7, 5, 4
    vol = blob_density(W, H, D, seed=5)
    cam = (orbit_camera(11, 9, W, H, D, steps=10) if orbit else capi.default_camera(11, 9, W, H, D))
    cam.steps = 10
    cam.focal = 6.0   # wide view: the box covers the centre, the corners miss
    img = oracle32.render(vol, cam)
    pixels = [(0, 0), (5, 4), (3, 6), (10, 8), (7, 2), (1, 7)]
    hits = 0
    for px, py in pixels:
        ref = shader_pixel(vol, cam, px, py)
        np.testing.assert_array_equal(img[py, px, :3], ref[:3], err_msg=str((px, py)))
        np.testing.assert_allclose(img[py, px, 3], ref[3], rtol=ALPHA_RTOL)
        hits += int(ref[3] < 1)
    assert 0 < hits < len(pixels)   # both hits and misses were checked


def test_oracle_scaling_and_misses(oracle32):
    W, H, D = 12, 10, 8
    vol = blob_density(W, H, D)
    cam = orbit_camera(24, 20, W, H, D, steps=30)
    cam.focal = 14.0
    a = oracle32.render(vol, cam)
    b = oracle32.render(2 * vol, cam)
    np.testing.assert_array_equal(b[..., :3], 2 * a[..., :3])      # scaling by 2 is exact through every lerp
    miss = a[..., 3] == 1
    assert miss.any() and (~miss).any()
    assert not a[miss][:, :3].any()
    z = oracle32.render(np.zeros_like(vol), cam)
    np.testing.assert_array_equal(z[..., :3], 0)
    np.testing.assert_array_equal(z[..., 3], 1)


@pytest.mark.gpu
@pytest.mark.parametrize("orbit", [False, True])
def test_render_matches_oracle(zqs_lib, oracle32, orbit):
    torch = pytest.importorskip("torch")
    W, H, D = 40, 32, 24
    vol = blob_density(W, H, D)
    cam = orbit_camera(96, 72, W, H, D) if orbit else capi.default_camera(96, 72, W, H, D)
    cam.steps = 64
    cam.focal = 60.0
    dv = torch.from_numpy(vol).cuda()
    out = torch.empty((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
    capi.render_density(dv.data_ptr(), W, H, D, cam, out.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    img = out.cpu().numpy()
    ref = oracle32.render(vol, cam)
    assert_image_equal(img, ref)
    assert (ref[..., 3] < 1).sum() > 100 and (ref[..., 3] == 1).sum() > 100


@pytest.mark.gpu
def test_grid_render_matches_oracle(zqs_lib, oracle32):
    torch = pytest.importorskip("torch")
    W, H, D = 32, 28, 24
    w = wl.small_case(W, H, D, K=15, vel_amp=0.2)
    g = capi.Grid(W, H, D)
    g.set_params(w.params)
    g.load_state(w.occ, w.u, w.v, w.w, w.T, w.rho)
    g.step(4)
    rho = g.download(capi.FIELD_DENSITY)
    assert rho.any()
    cam = orbit_camera(64, 48, W, H, D, steps=80, scale=4.0)
    cam.focal = 40.0
    out = torch.empty((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
    g.render(cam, out.data_ptr())
    g.sync()
    assert_image_equal(out.cpu().numpy(), oracle32.render(rho, cam))
    g.close()


@pytest.mark.gpu
def test_render_full_size_properties(zqs_lib):
    """The viewer's default view (1024x768, 300 samples) of a 256^3 volume:
    doubling the density doubles RGB bit for bit, misses are (0, 0, 0, 1)."""
    torch = pytest.importorskip("torch")
    N = 256
    gen = torch.Generator(device="cuda").manual_seed(7)
    vol = torch.rand((N, N, N), generator=gen, device="cuda", dtype=torch.float32)
    cam = capi.default_camera(1024, 768, N, N, N)
    a = torch.empty((768, 1024, 4), dtype=torch.float32, device="cuda")
    b = torch.empty_like(a)
    s = torch.cuda.current_stream().cuda_stream
    capi.render_density(vol.data_ptr(), N, N, N, cam, a.data_ptr(), s)
    vol2 = vol * 2
    capi.render_density(vol2.data_ptr(), N, N, N, cam, b.data_ptr(), s)
    torch.cuda.synchronize()
    assert torch.equal(b[..., :3], 2 * a[..., :3])
    miss = a[..., 3] == 1
    assert bool(miss.any()) and bool((~miss).any())
    assert not bool(a[miss][:, :3].any())
    # a ray through the middle of the box sees about one box depth of mean density 0.5
    mid = float(a[384, 512, 0])
    assert 0.4 < mid < 0.6, mid


@pytest.mark.gpu
def test_render_argument_checks(zqs_lib):
    torch = pytest.importorskip("torch")
    vol = torch.zeros((4, 4, 4), device="cuda")
    out = torch.empty((8 * 8 * 4 + 1,), device="cuda")
    cam = capi.default_camera(8, 8, 4, 4, 4)
    for bad in ("steps", "width"):
        c = capi.default_camera(8, 8, 4, 4, 4)
        setattr(c, bad, -1)
        with pytest.raises(capi.ZQSError) as e:
            capi.render_density(vol.data_ptr(), 4, 4, 4, c, out.data_ptr())
        assert e.value.code == capi.ZQS_EINVAL
    with pytest.raises(capi.ZQSError) as e:      # RGBA is written as float4: 16-byte alignment
        capi.render_density(vol.data_ptr(), 4, 4, 4, cam, out.data_ptr() + 4)
    assert e.value.code == capi.ZQS_EINVAL
    capi.render_density(vol.data_ptr(), 4, 4, 4, cam, out.data_ptr())
    torch.cuda.synchronize()
