"""GPU renders against the converged FP64 references: the CUDA path is an unbiased
estimator of the same image (mean error within a few standard errors) and its RMSE,
trimmed of the 1% firefly pixels, halves when the passes quadruple."""
import numpy as np
import pytest

from yune_gb300 import quality, scenes
from yune_gb300.core import Renderer

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,passes", [("c0", 64), ("c0_bdpt", 16)])
def test_gpu_render_converges_to_fp64_reference(name, passes):
    s = scenes.CONFIGS[name]()
    ref = quality.load_reference(name)
    seeds = scenes.pass_seeds(5, 4 * passes)
    with Renderer(0) as r:
        sid = r.upload(s)
        r.set_camera(s.cam)
        aid = r.alloc_accum(s.width, s.height)
        r.render_passes(sid, aid, seeds[:passes], reset_first=1, cfg=s.cfg)
        trim1 = quality.trimmed_rmse(r.read_accum(aid), ref)
        r.render_passes(sid, aid, seeds[passes:], reset_first=0, cfg=s.cfg)
        img = r.read_accum(aid)
        rmse4, rel4, bias4 = quality.error(img, ref)
        trim4 = quality.trimmed_rmse(img, ref)
    assert np.all(img[..., 3] == 4 * passes)
    assert abs(bias4) < 5.0 * rmse4 / np.sqrt(len(ref["xs"]))
    assert 1.5 < trim1 / trim4 < 2.7   # 1/sqrt(passes): 2 expected
