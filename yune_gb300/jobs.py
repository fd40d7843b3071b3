"""Render jobs described as JSON: the scene, the frame, the pass count and the options
the reference fixes with #defines in its kernel text (udpt.cl:3-9, bdpt.cl:1-8) or
with GUI state (src/RendererGUI.cpp:44-66: GI on/off, BVH bins), in one document.

    {
      "scene": {"config": "c1", "params": {"level": 5}},   # a configuration of scenes.CONFIGS
               # or {"obj": "model.obj", "bins": 20, "leaf": 10}   (Scene::loadModel)
      "cache": "c1_l5.ysc",          # optional: binary scene cache file (configurations only)
      "width": 512, "height": 512,   # optional: the configuration's frame otherwise
      "spp": 64,                     # passes
      "seed": 0,                     # per-pass rand values: std::mt19937(seed)
      "gi": true,                    # GI_CHECK (udpt.cl:158)
      "integrator": "udpt",          # "udpt", "bdpt" or "bdpt_mis"
      "mis": true, "rr_threshold": 3, "max_depth": 16, "brdf": "oren_nayar",
      "mis_lobe_fix": true, "bdpt_bounces": 8
    }

Every key but "scene" is optional; options left out keep the scene's own configuration.
Unknown keys and out-of-range values raise ValueError naming them, so a mistyped option
never falls back silently.
"""
import json
import os
from dataclasses import dataclass, replace

from . import scenes

INTEGRATORS = {"udpt": 0, "bdpt": 1, "bdpt_mis": 2}
BRDFS = {"lambert": 0, "oren_nayar": 1}
KEYS = {"scene", "cache", "width", "height", "spp", "seed", "gi", "integrator", "mis", "rr_threshold", "max_depth",
        "brdf", "mis_lobe_fix", "bdpt_bounces"}


@dataclass
class Job:
    scene: scenes.SceneData   # arrays, frame size, pass count and pass options (scene.cfg)
    seeds: object             # one rand value per pass (uint32 array)
    gi_check: int


def _int(doc, key, lo, hi):
    v = doc[key]
    if isinstance(v, bool) or not isinstance(v, int) or not lo <= v <= hi:
        raise ValueError("job: %r must be an integer in [%d, %d], got %r" % (key, lo, hi, v))
    return v


def _bool(doc, key):
    v = doc[key]
    if not isinstance(v, bool):
        raise ValueError("job: %r must be true or false, got %r" % (key, v))
    return int(v)


def _choice(doc, key, table):
    v = doc[key]
    if v not in table:
        raise ValueError("job: %r must be one of %s, got %r" % (key, sorted(table), v))
    return table[v]


def from_dict(doc, base_dir="."):
    """The Job a JSON document describes (relative file names resolve against base_dir)."""
    if not isinstance(doc, dict):
        raise ValueError("job: the document must be an object")
    unknown = sorted(set(doc) - KEYS)
    if unknown:
        raise ValueError("job: unknown keys %s" % unknown)
    if "scene" not in doc or not isinstance(doc["scene"], dict):
        raise ValueError("job: 'scene' must be an object")
    sc = doc["scene"]
    size = {}
    if "width" in doc:
        size["width"] = _int(doc, "width", 1, 16384)
    if "height" in doc:
        size["height"] = _int(doc, "height", 1, 16384)
    if "config" in sc:
        if set(sc) - {"config", "params"}:
            raise ValueError("job: unknown scene keys %s" % sorted(set(sc) - {"config", "params"}))
        name = sc["config"]
        if name not in scenes.CONFIGS:
            raise ValueError("job: scene config must be one of %s, got %r" % (sorted(scenes.CONFIGS), name))
        params = sc.get("params", {})
        if not isinstance(params, dict):
            raise ValueError("job: scene params must be an object")
        params = dict(params, **size)
        if "cache" in doc:
            s = scenes.cached(name, os.path.join(base_dir, doc["cache"]), **params)
        else:
            s = scenes.CONFIGS[name](**params)
    elif "obj" in sc:
        if set(sc) - {"obj", "bins", "leaf"}:
            raise ValueError("job: unknown scene keys %s" % sorted(set(sc) - {"obj", "bins", "leaf"}))
        if "cache" in doc:
            raise ValueError("job: 'cache' applies to scene configurations only")
        bins = _int(sc, "bins", 0, 256) if "bins" in sc else 20
        leaf = _int(sc, "leaf", 1, 10) if "leaf" in sc else 10
        s = scenes.from_obj(os.path.join(base_dir, sc["obj"]), bins=bins, leaf=leaf, **size)
    else:
        raise ValueError("job: 'scene' needs 'config' or 'obj'")
    cfg = dict(s.cfg)
    if "integrator" in doc:
        cfg["integrator"] = _choice(doc, "integrator", INTEGRATORS)
    if "mis" in doc:
        cfg["mis"] = _bool(doc, "mis")
    if "rr_threshold" in doc:
        cfg["rr_threshold"] = _int(doc, "rr_threshold", 0, 100000)
    if "max_depth" in doc:
        cfg["max_depth"] = _int(doc, "max_depth", 0, 100000)
    if "brdf" in doc:
        cfg["brdf_model"] = _choice(doc, "brdf", BRDFS)
    if "mis_lobe_fix" in doc:
        cfg["mis_lobe_fix"] = _bool(doc, "mis_lobe_fix")
    if "bdpt_bounces" in doc:
        # the range yc_render_pass accepts (2..32; 3..32 with YC_BDPT_MIS)
        cfg["bdpt_bounces"] = _int(doc, "bdpt_bounces", 3 if cfg["integrator"] == 2 else 2, 32)
    spp = _int(doc, "spp", 1, 1 << 24) if "spp" in doc else s.spp
    seed = _int(doc, "seed", 0, 0xFFFFFFFF) if "seed" in doc else 0
    gi = _bool(doc, "gi") if "gi" in doc else 1
    s = replace(s, cfg=cfg, spp=spp)
    return Job(s, scenes.pass_seeds(seed, spp), gi)


def load(path):
    """The Job of a JSON file."""
    with open(path) as f:
        doc = json.load(f)
    return from_dict(doc, os.path.dirname(os.path.abspath(path)))

