"""Generates the golden fixtures in this directory from Yune's own code, compiled as C++
by oracle/build_oracle.py (needs the reference tree; run where it is present):

    python tests/golden/make_golden.py

The fixtures pin the CPU oracle and the host producers on machines without the
reference tree:
  bvh_<scene>.npz      BVH::createBVH node arrays (src/BVH.cpp) for the scene's triangles
  trace_<scene>.npz    traceRay (kernels/legacy/udpt.cl:240-286) on seeded rays
                       (oracle_py.seeded_rays(scene, 4096, seed=5)) and on the segments
                       ending just past each closest hit (shadow rays)
  render_c0.npz        3 passes of `pathtracer` (udpt.cl as shipped, and with -DMIS
                       RR_THRESHOLD 3) on a 32x24 Cornell box, plus `tonemap`
                       (kernels/post-proc/tonemap.cl) of the MIS accumulator
  oren_nayar.npz       OrenNayarBRDF (kernels/legacy/udpt-primitives.cl:696-725)
  render_bdpt.npz      2 passes of the BDPT `pathtracer` (kernels/legacy/bdpt.cl with
                       BDPT_BOUNCES 8) on a 32x24 Cornell box with 1 and with 4 lights
  obj_test_scene.npz   Scene::loadModel (src/Scene.cpp:133-383) on the loader test files
                       of obj_files.py: triangles, materials and the BVH node array
  obj_cornellbox.npz   the same on the reference's geometry/cornellbox.obj (the test
                       that uses it needs that file and skips without it)
  render_variant_b.npz passes of udpt.cl -DMIS with the Oren-Nayar diffuse rule of
                       udpt-primitives.cl (the configurations' composite; oracle/_ref variant
                       udpt_mis_on) on the 32x24 Cornell box (3 passes, roulette after
                       bounce 3) and on the level-3 glass scene (2 passes, at most 16
                       bounces); python tests/golden/make_golden.py variant_b writes this
                       file alone
  bvh_large.npz        SHA-256 digests of BVH::createBVH node arrays for a 327,714-
                       triangle scene (c1 with a level-7 icosphere) at leaf sizes 4 and
                       10: large enough for the host builder to split single nodes
                       over threads (python tests/golden/make_golden.py large writes
                       this file alone)
Each file records a SHA-256 of the scene arrays it was made from.
"""
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle_py as O  # noqa: E402
from yune_gb300 import scenes  # noqa: E402
from yune_gb300.layouts import MATERIAL  # noqa: E402


def scene_hash(s):
    h = hashlib.sha256()
    for a in (s.tris, s.mats, s.lights, s.cam):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def golden_scenes():
    return {"c0": scenes.c0(32, 24), "c1l3": scenes.c1(32, 24, level=3)}


def node_fields(nodes):
    return dict(p_min=nodes["p_min"][:, :3].copy(), p_max=nodes["p_max"][:, :3].copy(),
                child_idx=nodes["child_idx"].copy(), vert_len=nodes["vert_len"].copy(),
                vert_list=np.where(np.arange(10)[None, :] < np.maximum(nodes["vert_len"], 0)[:, None],
                                   nodes["vert_list"], -1).astype(np.int32))


def node_digest(nodes):
    """SHA-256 of node_fields(nodes), the fields in a fixed order."""
    h = hashlib.sha256()
    f = node_fields(nodes)
    for k in ("p_min", "p_max", "child_idx", "vert_len", "vert_list"):
        h.update(np.ascontiguousarray(f[k]).tobytes())
    return h.hexdigest()


LARGE_LEAVES = (4, 10)


def large_scene():
    return scenes.c1(16, 16, level=7)


def make_large():
    s = large_scene()
    out = {"scene_sha256": scene_hash(s), "bins": 20, "leaves": np.array(LARGE_LEAVES, np.int32)}
    for leaf in LARGE_LEAVES:
        nodes = O.ref_bvh(s.tris, 20, leaf)
        out["nodes_leaf%d" % leaf] = np.int64(len(nodes))
        out["digest_leaf%d" % leaf] = node_digest(nodes)
    np.savez_compressed(os.path.join(HERE, "bvh_large.npz"), **out)


TRI_FIELDS = ("v1", "v2", "v3", "vn1", "vn2", "vn3", "matID")


def obj_fields(tris, mats, nodes, no_normals=()):
    """The loader's output as comparable arrays (padding bytes and vert_list entries past
    a leaf's count, which the reference leaves unset, are dropped; so are the normals of
    the triangles in no_normals, faces without normal indices, written as zeros)."""
    out = {"tri_" + k: np.ascontiguousarray(tris[k]) for k in TRI_FIELDS}
    for k in ("vn1", "vn2", "vn3"):
        out["tri_" + k][list(no_normals)] = 0.0
    out["mats"] = np.ascontiguousarray(mats).view(np.uint8).reshape(len(mats), -1)
    out.update({"node_" + k: v for k, v in node_fields(nodes).items()})
    return out


VARIANT_B = {"c0": dict(rr=3, max_depth=100000, passes=3, seed=2025),
             "c1l3": dict(rr=3, max_depth=16, passes=2, seed=2026)}


def make_variant_b():
    out = {}
    for name, s in golden_scenes().items():
        v = VARIANT_B[name]
        seeds = scenes.pass_seeds(v["seed"], v["passes"])
        acc = np.zeros((24, 32, 4), np.float32)
        for k, sd in enumerate(seeds):
            O.ref_render(s, acc, sd, 1 if k == 0 else 0, "udpt_mis_on", v["rr"], v["max_depth"])
        out[name] = acc
        out[name + "_seeds"] = seeds
        out[name + "_sha256"] = scene_hash(s)
    np.savez_compressed(os.path.join(HERE, "render_variant_b.npz"), **out)


def main():
    if O.ref() is None:
        raise SystemExit("the compiled reference is not available here")
    import tempfile
    sys.path.insert(0, HERE)
    import obj_files
    from oracle import build_oracle
    with tempfile.TemporaryDirectory() as d:
        np.savez_compressed(os.path.join(HERE, "obj_test_scene.npz"),
                            **obj_fields(*O.ref_load_obj(obj_files.write(d)), no_normals=obj_files.NO_NORMALS))
    np.savez_compressed(os.path.join(HERE, "obj_cornellbox.npz"),
                        **obj_fields(*O.ref_load_obj(os.path.join(build_oracle.reference_tree(), "geometry", "cornellbox.obj"))))
    for name, s in golden_scenes().items():
        leaf = 10 if name == "c0" else 4
        nodes = O.ref_bvh(s.tris, 20, leaf)
        np.savez_compressed(os.path.join(HERE, "bvh_%s.npz" % name), scene_sha256=scene_hash(s), bins=20, leaf=leaf,
                            **node_fields(nodes))
        rays = O.seeded_rays(s, 4096, seed=5)
        tri, light, t = O.ref_trace(s, rays)
        seg = rays.copy()
        seg[:, 8] = np.where(np.isfinite(t), t * np.float32(1.001), np.float32(0.6))
        occ_tri, occ_light, _ = O.ref_trace(s, seg, any_hit=True)
        np.savez_compressed(os.path.join(HERE, "trace_%s.npz" % name), scene_sha256=scene_hash(s), ray_seed=5,
                            n_rays=4096, tri=tri, light=light, t=t, occluded=((occ_tri >= 0) | (occ_light >= 0)))
    s = golden_scenes()["c0"]
    seeds = scenes.pass_seeds(2024, 3)
    out = {}
    for variant, rr in (("udpt_a", 6), ("udpt_mis", 3)):
        acc = np.zeros((24, 32, 4), np.float32)
        for k, sd in enumerate(seeds):
            O.ref_render(s, acc, sd, 1 if k == 0 else 0, variant, rr, 100000)
        out[variant] = acc
    out["tonemap_mis"] = O.ref_tonemap(out["udpt_mis"])
    np.savez_compressed(os.path.join(HERE, "render_c0.npz"), scene_sha256=scene_hash(s), seeds=seeds, **out)
    # Oren-Nayar on random frames
    rng = np.random.default_rng(9)
    n = 256
    nrm = rng.normal(size=(n, 3))
    nrm /= np.linalg.norm(nrm, axis=1, keepdims=True)
    wi = rng.normal(size=(n, 3))
    wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    wo = rng.normal(size=(n, 3))
    wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    hp = rng.uniform(-0.5, 0.5, size=(n, 3))
    m = np.zeros(1, MATERIAL)
    m["kd"] = (0.63, 0.065, 0.05, 1.0)
    m["alpha_x"] = 0.09
    f4 = lambda v, w: np.concatenate([v, np.full((n, 1), w)], axis=1).astype(np.float32)  # noqa: E731
    NRM, WI, WO, HP = f4(nrm, 0.0), f4(wi, 0.0), f4(wo, 0.0), f4(hp, 1.0)
    res = np.zeros((n, 4), np.float32)
    for i in range(n):
        o = np.zeros(4, np.float32)
        O.ref().ref_oren_nayar(m.ctypes.data, HP[i].ctypes.data, NRM[i].ctypes.data, WI[i].ctypes.data,
                               WO[i].ctypes.data, o.ctypes.data)
        res[i] = o
    np.savez_compressed(os.path.join(HERE, "oren_nayar.npz"), material=m, normal=NRM, w_i=WI, w_o=WO, hit_point=HP,
                        value=res)
    # BDPT
    out = {}
    seeds = scenes.pass_seeds(606, 2)
    for lights, variant in ((1, "bdpt8"), (4, "bdpt8_l4")):
        sb = scenes.c0_bdpt(32, 24, bounces=8, lights=lights)
        acc = np.zeros((24, 32, 4), np.float32)
        for k, sd in enumerate(seeds):
            O.ref_render(sb, acc, sd, 1 if k == 0 else 0, variant, 4, 100000)
        out["lights%d" % lights] = acc
        out["sha_lights%d" % lights] = scene_hash(sb)
    np.savez_compressed(os.path.join(HERE, "render_bdpt.npz"), seeds=seeds, **out)
    make_large()
    make_variant_b()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "large":
        if O.ref() is None:
            raise SystemExit("the compiled reference is not available here")
        make_large()
    elif len(sys.argv) > 1 and sys.argv[1] == "variant_b":
        if O.ref() is None:
            raise SystemExit("the compiled reference is not available here")
        make_variant_b()
    else:
        main()
