"""Render jobs from JSON (yune_gb300.jobs): scene, frame, passes and the pass options the
reference fixes with #defines (udpt.cl:3-9, bdpt.cl:1-8) map onto SceneData and
yc_pass_cfg fields; unknown keys and bad values are refused by name. CPU only."""
import json
import os
import sys

import numpy as np
import pytest

from yune_gb300 import jobs, scenes

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _write(tmp_path, doc, name="job.json"):
    p = tmp_path / name
    p.write_text(json.dumps(doc))
    return str(p)


def test_configuration_job_with_every_option(tmp_path):
    doc = {"scene": {"config": "c1", "params": {"level": 3, "seed": 2}}, "width": 40, "height": 30, "spp": 5,
           "seed": 9, "gi": False, "integrator": "udpt", "mis": False, "rr_threshold": 6, "max_depth": 12,
           "brdf": "lambert", "mis_lobe_fix": False}
    job = jobs.load(_write(tmp_path, doc))
    s = job.scene
    ref = scenes.c1(40, 30, level=3, seed=2)
    assert s.tris.tobytes() == ref.tris.tobytes() and s.nodes.tobytes() == ref.nodes.tobytes()
    assert (s.width, s.height, s.spp) == (40, 30, 5)
    assert s.cfg == dict(ref.cfg, integrator=0, mis=0, rr_threshold=6, max_depth=12, brdf_model=0, mis_lobe_fix=0)
    assert np.array_equal(job.seeds, scenes.pass_seeds(9, 5)) and job.gi_check == 0


def test_defaults_keep_the_configuration():
    job = jobs.from_dict({"scene": {"config": "c0_bdpt", "params": {"width": 16, "height": 16}}})
    ref = scenes.c0_bdpt(16, 16)
    assert job.scene.cfg == ref.cfg and job.scene.spp == ref.spp and job.gi_check == 1
    assert np.array_equal(job.seeds, scenes.pass_seeds(0, ref.spp))
    job = jobs.from_dict({"scene": {"config": "c0_bdpt", "params": {"width": 16, "height": 16}},
                          "integrator": "bdpt_mis", "bdpt_bounces": 6})
    assert job.scene.cfg["integrator"] == 2 and job.scene.cfg["bdpt_bounces"] == 6


def test_obj_job(tmp_path):
    sys.path.insert(0, GOLD)
    try:
        import obj_files
    finally:
        sys.path.remove(GOLD)
    obj = obj_files.write(str(tmp_path))
    doc = {"scene": {"obj": os.path.basename(obj), "bins": 7, "leaf": 8}, "width": 24, "height": 20, "spp": 2}
    job = jobs.load(_write(tmp_path, doc))      # the OBJ name resolves against the job file's folder
    ref = scenes.from_obj(obj, width=24, height=20, bins=7, leaf=8)
    assert job.scene.tris.tobytes() == ref.tris.tobytes() and job.scene.nodes.tobytes() == ref.nodes.tobytes()
    assert job.scene.cfg == ref.cfg and job.scene.spp == 2


def test_cached_job_reads_the_scene_back(tmp_path, monkeypatch):
    doc = {"scene": {"config": "c0", "params": {"seed": 1}}, "width": 16, "height": 16, "cache": "c0.ysc"}
    p = _write(tmp_path, doc)
    a = jobs.load(p)
    assert (tmp_path / "c0.ysc").exists()
    calls = []
    real = scenes.CONFIGS["c0"]
    monkeypatch.setitem(scenes.CONFIGS, "c0", lambda **kw: calls.append(kw) or real(**kw))
    b = jobs.load(p)
    assert calls == []
    assert a.scene.tris.tobytes() == b.scene.tris.tobytes() and a.scene.cfg == b.scene.cfg


@pytest.mark.parametrize("doc,word", [
    ({"scene": {"config": "c0"}, "sppp": 4}, "unknown keys"),
    ({"spp": 4}, "'scene'"),
    ({"scene": {"config": "c9"}}, "scene config"),
    ({"scene": {"config": "c0", "extra": 1}}, "unknown scene keys"),
    ({"scene": {"config": "c0", "params": [1]}}, "params"),
    ({"scene": {"config": "c0"}, "integrator": "path"}, "'integrator'"),
    ({"scene": {"config": "c0"}, "mis": 1}, "'mis'"),
    ({"scene": {"config": "c0"}, "spp": True}, "'spp'"),
    ({"scene": {"config": "c0"}, "spp": 0}, "'spp'"),
    ({"scene": {"config": "c0"}, "width": 2.5}, "'width'"),
    ({"scene": {"config": "c0"}, "brdf": "phong"}, "'brdf'"),
    ({"scene": {"config": "c0"}, "integrator": "bdpt_mis", "bdpt_bounces": 2}, "'bdpt_bounces'"),
    ({"scene": {"config": "c0"}, "bdpt_bounces": 33}, "'bdpt_bounces'"),
    ({"scene": {"obj": "x.obj"}, "cache": "x.ysc"}, "'cache'"),
    ({"scene": {"obj": "x.obj", "leaf": 11}}, "'leaf'"),
    ({"scene": {}}, "'config' or 'obj'"),
    ([1, 2], "object"),
])
def test_bad_documents_are_refused_by_name(doc, word):
    with pytest.raises(ValueError) as e:
        jobs.from_dict(doc)
    assert word in str(e.value)
