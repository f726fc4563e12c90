"""Seeded synthetic session inputs for the five benchmark workloads.

The reference's own benchmarks use JPEG photos (lib/benches/all-the-things.rs);
here every input is generated from a seed, so the same workload can be rebuilt
on any machine with numpy alone.  A session spec is a plain dict:

    {"name", "out_w", "out_h",
     "params": {nearest_neighbors, random_sample_locations, cauchy_dispersion,
                backtrack_percent, backtrack_stages, seed, guide_alpha,
                tiling_mode, random_init (None or int)},
     "examples": [{"image": HxWx4 u8, "guide": HxWx4 u8 or None,
                   "sample": "all" | "ignore" | "image", "mask": HxWx4 u8}],
     "target_guide": HxWx4 u8 or None,
     "inpaint_mask": HxWx4 u8 or None, "inpaint_index": int}

Images are RGBA8 (alpha 255); guides are grey (R = G = B).
"""
import math

import numpy as np

DEFAULTS = dict(
    nearest_neighbors=50,
    random_sample_locations=50,
    cauchy_dispersion=1.0,
    backtrack_percent=0.5,
    backtrack_stages=5,
    seed=0,
    guide_alpha=0.8,
    tiling_mode=False,
    random_init=None,
)


def _bilinear_up(lat, h, w):
    """Bilinear upsampling of a (ch+1)x(cw+1) lattice onto an h x w grid."""
    ch, cw = lat.shape[0] - 1, lat.shape[1] - 1
    ys = (np.arange(h) + 0.5) / h * ch
    xs = (np.arange(w) + 0.5) / w * cw
    y0 = np.minimum(np.floor(ys).astype(np.int64), ch - 1)
    x0 = np.minimum(np.floor(xs).astype(np.int64), cw - 1)
    fy = (ys - y0)[:, None]
    fx = (xs - x0)[None, :]
    a = lat[y0][:, x0]
    b = lat[y0][:, x0 + 1]
    c = lat[y0 + 1][:, x0]
    d = lat[y0 + 1][:, x0 + 1]
    return (a * (1 - fx) + b * fx) * (1 - fy) + (c * (1 - fx) + d * fx) * fy


def value_noise(rng, h, w, octaves, base_cells=4):
    """Sum of bilinear-upsampled uniform lattices, octave i weighted 0.5**i,
    normalised to [0, 1]."""
    f = np.zeros((h, w), np.float64)
    for i in range(octaves):
        cells = base_cells * (2 ** i)
        lat = rng.random((cells + 1, cells + 1))
        f += (0.5 ** i) * _bilinear_up(lat, h, w)
    lo, hi = f.min(), f.max()
    return (f - lo) / (hi - lo if hi > lo else 1.0)


def texture(seed, h, w):
    """4-octave value noise mapped through a random 3-colour palette, plus 12
    random axis-aligned rectangles of uniform-random colour; alpha 255."""
    rng = np.random.default_rng(seed)
    t = value_noise(rng, h, w, 4)
    pal = rng.integers(0, 256, size=(3, 3)).astype(np.float64)
    lo = np.clip(t * 2.0, 0.0, 1.0)[..., None]
    hi = np.clip(t * 2.0 - 1.0, 0.0, 1.0)[..., None]
    rgb = np.where(t[..., None] < 0.5, pal[0] * (1 - lo) + pal[1] * lo, pal[1] * (1 - hi) + pal[2] * hi)
    img = np.zeros((h, w, 4), np.uint8)
    img[..., :3] = np.clip(np.floor(rgb + 0.5), 0, 255).astype(np.uint8)
    img[..., 3] = 255
    for _ in range(12):
        rw = int(rng.integers(max(1, w // 16), max(2, w // 4) + 1))
        rh = int(rng.integers(max(1, h // 16), max(2, h // 4) + 1))
        x0 = int(rng.integers(0, max(1, w - rw + 1)))
        y0 = int(rng.integers(0, max(1, h - rh + 1)))
        col = rng.integers(0, 256, size=3).astype(np.uint8)
        img[y0:y0 + rh, x0:x0 + rw, :3] = col
    return img


def _gauss_kernel(sigma):
    r = int(math.ceil(3 * sigma))
    k = np.array([math.exp(-(i * i) / (2.0 * sigma * sigma)) for i in range(-r, r + 1)], np.float64)
    return k / k.sum()


def gaussian_blur(f, sigma):
    """Separable Gaussian blur of a 2-D float field, edge-replicated."""
    k = _gauss_kernel(sigma)
    r = len(k) // 2
    p = np.pad(f, ((0, 0), (r, r)), mode="edge")
    g = np.zeros_like(f)
    for i, kv in enumerate(k):
        g += kv * p[:, i:i + f.shape[1]]
    p = np.pad(g, ((r, r), (0, 0)), mode="edge")
    out = np.zeros_like(f)
    for i, kv in enumerate(k):
        out += kv * p[i:i + f.shape[0], :]
    return out


def grey_rgba(v):
    v = np.clip(np.floor(v + 0.5), 0, 255).astype(np.uint8)
    img = np.empty(v.shape + (4,), np.uint8)
    img[..., 0] = v
    img[..., 1] = v
    img[..., 2] = v
    img[..., 3] = 255
    return img


def example_guide(seed, h, w, sigma=8.0):
    """2-octave value noise, Gaussian-blurred, thresholded at its median."""
    rng = np.random.default_rng(seed)
    f = gaussian_blur(value_noise(rng, h, w, 2), sigma)
    return grey_rgba(np.where(f > np.median(f), 255.0, 0.0))


def target_guide(seed, h, w, ndiscs=3, rmin=60, rmax=160, sigma=12.0):
    """Union of random discs, Gaussian-blurred (radii scale with the side)."""
    rng = np.random.default_rng(seed)
    s = min(h, w) / 512.0
    yy, xx = np.mgrid[0:h, 0:w]
    m = np.zeros((h, w), np.float64)
    for _ in range(ndiscs):
        r = rng.uniform(rmin * s, rmax * s)
        cy, cx = rng.uniform(0, h), rng.uniform(0, w)
        m = np.maximum(m, ((yy - cy) ** 2 + (xx - cx) ** 2 <= r * r).astype(np.float64))
    return grey_rgba(gaussian_blur(m * 255.0, max(1.0, sigma * s)))


def _spec(name, w, h, examples, **params):
    p = dict(DEFAULTS)
    p.update(params)
    return {"name": name, "out_w": w, "out_h": h, "params": p, "examples": examples,
            "target_guide": None, "inpaint_mask": None, "inpaint_index": -1}


def config0(out=256, ex=128):
    """Plain single-example synthesis: 128^2 example (seed 0) -> 256^2."""
    return _spec("single_example_%d" % out, out, out, [{"image": texture(0, ex, ex)}], seed=0, random_init=0)


def config1(out=512, ex=300):
    """Multi-example remix: 4 x 300^2 examples (seeds 1-4), random_init 10,
    seed 211, tiling, 512^2 output."""
    exs = [{"image": texture(s, ex, ex)} for s in (1, 2, 3, 4)]
    return _spec("multi_example_tiling_%d" % out, out, out, exs, seed=211, random_init=10, tiling_mode=True)


def config2(out=512, ex=256):
    """Guided synthesis: 256^2 example with a grey guide, 512^2 target guide,
    alpha 0.8, seed 7."""
    e = {"image": texture(2, ex, ex), "guide": example_guide(12, ex, ex)}
    s = _spec("guided_%d" % out, out, out, [e], seed=7, guide_alpha=0.8)
    s["target_guide"] = target_guide(22, out, out)
    return s


def _logu(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def config3_sessions(n=64, seed=3, scale=1.0):
    """Batched mix: example sides log-uniform 64-512, outputs 128-1024,
    k and m from {8, 20, 50}, a quarter guided; per-session seeds 1000+i.
    scale < 1 shrinks every side for quick tests."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        es = max(8, int(_logu(rng, 64, 512) * scale))
        os_ = max(8, int(_logu(rng, 128, 1024) * scale))
        k = int(rng.choice([8, 20, 50]))
        m = int(rng.choice([8, 20, 50]))
        guided = (i % 4) == 3
        e = {"image": texture(1000 + i, es, es)}
        if guided:
            e["guide"] = example_guide(5000 + i, es, es, sigma=max(1.0, 8.0 * es / 256))
        s = _spec("batch_%02d" % i, os_, os_, [e], seed=1000 + i, nearest_neighbors=k, random_sample_locations=m)
        if guided:
            s["target_guide"] = target_guide(6000 + i, os_, os_)
        out.append(s)
    return out


def inpaint_session(seed, side=512, scale=1.0):
    """Inpainting request: a side^2 example with 1-5 random rectangles
    covering 10-40% of it masked out (R < 255 = to be synthesised)."""
    rng = np.random.default_rng(seed)
    side = max(16, int(side * scale))
    img = texture(seed, side, side)
    mask = np.full((side, side, 4), 255, np.uint8)
    target = rng.uniform(0.10, 0.40) * side * side
    nrect = int(rng.integers(1, 6))
    for _ in range(nrect):
        a = target / nrect
        rw = int(np.clip(math.sqrt(a) * rng.uniform(0.6, 1.6), 2, side))
        rh = int(np.clip(a / rw, 2, side))
        x0 = int(rng.integers(0, side - rw + 1))
        y0 = int(rng.integers(0, side - rh + 1))
        mask[y0:y0 + rh, x0:x0 + rw, :3] = 0
    s = _spec("inpaint_%d" % seed, side, side, [{"image": img}], seed=seed)
    s["inpaint_mask"] = mask
    s["inpaint_index"] = 0
    return s


def config4_requests(n, lam, seed=4, scale=1.0, mix_seed=3):
    """Poisson request stream: arrival times (s) with rate lam and a session
    spec per request drawn from the batched mix (70%) or inpainting (30%)."""
    rng = np.random.default_rng(seed)
    mix = config3_sessions(64, seed=mix_seed, scale=scale)
    t = 0.0
    reqs = []
    for i in range(n):
        t += rng.exponential(1.0 / lam)
        if rng.random() < 0.3:
            s = inpaint_session(7000 + i, scale=scale)
        else:
            s = mix[int(rng.integers(0, len(mix)))]
        reqs.append((t, s))
    return reqs


def by_name(name, **kw):
    return {"config0": config0, "config1": config1, "config2": config2}[name](**kw)
