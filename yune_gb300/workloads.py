"""Seeded mixed workloads for the batch and serving engine.

c2_jobs      the batched configuration: Cornell boxes plus N displaced icospheres with a
             total triangle count log-uniform in [1k, 500k], vertex displacement
             uniform +-5% of the radius, one material per sphere drawn uniformly from
             {Oren-Nayar, modified Phong with exponent in [10, 200], dielectric with IOR
             in [1.3, 1.7]}, resolution drawn from {256^2, 512^2, 1280x720, 1920x1080}.
c3_scenes    the serving configuration's resident pool: scenes built the same way with
             10k..2M triangles.
c3_requests  Poisson arrivals; each request picks a resident scene and draws its
             resolution and target spp log-uniformly.
All draws come from numpy's PCG64 stream of the given seed.
"""
import math

import numpy as np

from . import scenes

RESOLUTIONS = [(256, 256), (512, 512), (1280, 720), (1920, 1080)]


def _sphere_levels(total, rng, max_level=7):
    """Icosphere levels whose triangle counts (20 * 4^level) add up to about `total`."""
    levels = []
    remaining = total
    while remaining >= 320 or not levels:
        lv = max(2, min(max_level, int(math.floor(math.log(max(remaining, 320) / 20.0, 4)))))
        levels.append(lv)
        remaining -= 20 * 4 ** lv
        if len(levels) >= 24:
            break
    return levels


def random_material(rng):
    kind = int(rng.integers(0, 3))
    if kind == 0:   # Oren-Nayar, sigma^2 in alpha_x
        c = rng.uniform(0.2, 0.85, 3)
        return scenes.material(kd=tuple(c), alpha=float(rng.uniform(0.0, 0.25)))
    if kind == 1:   # modified Phong
        e = float(rng.uniform(10, 200))
        c = rng.uniform(0.1, 0.45, 3)
        return scenes.material(kd=tuple(c), ks=(0.4, 0.4, 0.4), px=e / 2, py=e / 2, alpha=0.0)
    return scenes.dielectric(float(rng.uniform(1.3, 1.7)))


def mixed_scene(total_tris, seed, width, height, spp, cfg=None):
    rng = np.random.default_rng(seed)
    b = scenes.Builder().cornell(seed=seed)
    for i, lv in enumerate(_sphere_levels(total_tris, rng)):
        mid = b.add_material(random_material(rng))
        r = float(rng.uniform(0.06, 0.2))
        c = rng.uniform(-0.45 + r, 0.45 - r, 3)
        b.icosphere(tuple(c), r, lv, mid, disp=0.05, seed=seed * 1000 + i)
    tris, mats, lights = b.arrays()
    nodes, depth = scenes.build_bvh(tris, 20, 4)
    return scenes.SceneData(tris, mats, lights, nodes, depth, scenes.camera(), width, height, spp,
                            dict(cfg) if cfg else scenes.default_cfg(max_depth=16), "mixed")


CORNELL_TRIS = 34   # five walls (10 triangles) and two boxes (24)


def mixed_scene_tris(total_tris):
    """The triangle count of mixed_scene(total_tris, ...), without building it."""
    return CORNELL_TRIS + sum(20 * 4 ** lv for lv in _sphere_levels(total_tris, None))


def c2_specs(n_jobs=64, seed=0, max_tris=500_000):
    """(triangle target, scene seed, width, height) of each job of the mix."""
    rng = np.random.default_rng(seed)
    out = []
    for j in range(n_jobs):
        total = int(math.exp(rng.uniform(math.log(1000), math.log(max_tris))))
        w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
        out.append((total, seed * 100003 + j, w, h))
    return out


def c2_jobs(n_jobs=64, spp=64, seed=0, max_tris=500_000, cfg=None, only=None):
    """The mix's scenes; `only`: the indices of the jobs to build (all when None)."""
    specs = c2_specs(n_jobs, seed, max_tris)
    idx = range(n_jobs) if only is None else only
    return [mixed_scene(specs[j][0], specs[j][1], specs[j][2], specs[j][3], spp, cfg) for j in idx]


def c3_scenes(n_scenes=8, seed=1, min_tris=10_000, max_tris=2_000_000, only=None, cfg=None, width=256, height=256):
    """The serving pool's scenes; `only`: the indices of the scenes to build (all when None)."""
    rng = np.random.default_rng(seed)
    totals = [int(math.exp(rng.uniform(math.log(min_tris), math.log(max_tris)))) for _ in range(n_scenes)]
    idx = range(n_scenes) if only is None else only
    return [mixed_scene(totals[j], seed * 7919 + j, width, height, 1, cfg) for j in idx]


def c3_requests(n_requests, rate, n_scenes, seed=2, res_range=(256, 2048), spp_range=(16, 1024)):
    """(arrival_s, scene_index, width, height, spp) for n_requests Poisson arrivals."""
    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for _ in range(n_requests):
        t += float(rng.exponential(1.0 / rate))
        side = int(round(math.exp(rng.uniform(math.log(res_range[0]), math.log(res_range[1])))))
        spp = int(round(math.exp(rng.uniform(math.log(spp_range[0]), math.log(spp_range[1])))))
        out.append((t, int(rng.integers(0, n_scenes)), side, side, spp))
    return out
