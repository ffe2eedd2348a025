"""Every launch configuration of the 2D update kernels (warps per block and
copy-ring depth, the pairs the autotuner chooses among; forced with
AMR_GB300_STEP_CONFIG, read once per process) computes the same states: the
tuner's choice, which depends on the GPU's timings, never changes a result.

Each configuration runs in its own process: a 16x16-patch tree refined
uniformly to level 5 (1024 leaves), adapted by the gradient criterion
between levels 4 and 6 for 40 steps through the per-launch graph path (the
first interval on the same-level tree: multi-step passes, or the fused
interval in FP32; then one-step launches on the adapted tree), FP64 and
FP32.  Bar: final leaves and states bit-identical to the tuned run's."""
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, sys.argv[1])
import amr_gb300 as A
b = A.seeded_bumps(2, 3, 5, sigma=(0.03, 0.06))
out = []
for dt in (A.F64, A.F32):
    t = A.Tree(2, 16, 1, 7, capacity=20000, dtype=dt)
    t.refine_uniform(5)
    t.upload_state(A.gaussian_state(t.ids(), 2, 16, 1, 7, b, 1e-3, 7))
    st = t.run(40, 10, (0.8, -0.6), 0.4, "grad", 0.05, 0.01, 4, 6, per_launch=True)
    assert st["graph_intervals"] == 4 and st["remeshes_changed"] > 0
    out.append(t.ids().astype(np.float64))
    out.append(t.download_state().astype(np.float64).ravel())
np.save(sys.argv[2], np.concatenate(out))
"""

CONFIGS = ["", "4,2,0", "4,3,0", "8,1,0", "8,2,0", "8,3,0", "8,4,0", "16,2,0", "16,3,0", "16,4,0", "8,2,1"]


def test_launch_configurations_agree(tmp_path):
    pkg = str(Path(__file__).resolve().parents[1] / "gpu-amr_gb300")
    res = {}
    for cfg in CONFIGS:
        env = dict(os.environ)
        env.pop("AMR_GB300_STEP_CONFIG", None)
        if cfg:
            env["AMR_GB300_STEP_CONFIG"] = cfg
        out = tmp_path / f"c{cfg.replace(',', '_') or 'tuned'}.npy"
        subprocess.run([sys.executable, "-c", _SCRIPT, pkg, str(out)], env=env, check=True, timeout=600)
        res[cfg] = np.load(out)
    ref = res[""]
    for cfg, v in res.items():
        assert v.shape == ref.shape, cfg
        np.testing.assert_array_equal(v, ref, err_msg=cfg)
