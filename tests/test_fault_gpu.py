"""Failure detection without a GPU fault: a bounded wait that runs out returns an error
status to the host and leaves the context usable.  The guiding network's tensor-core
completion wait is made to run out by fault injection (spgpu_guiding_config
fault_injection: no MMA is issued, so nothing ever arrives on the mbarrier and the
wait, cut to 1024 polls, gives up); spgpu_guiding_mlp must return SPGPU_EKERNEL with
its message, and the same context must then evaluate the network correctly."""
import numpy as np
import pytest

from oracle import guide_oracle as go
from spica_gb300 import GpuBVHAccel, GpuGuide, scenes
from spica_gb300.gpu import SpgpuError

pytestmark = pytest.mark.gpu


def test_timed_out_tensor_core_wait_reports_and_context_survives(gpulib):
    import torch
    acc = GpuBVHAccel(scenes.box_room(width=8, height=8)).construct()
    rng = np.random.default_rng(3)
    x = rng.uniform(-1, 1, (300, 9)).astype(np.float32)
    feat = torch.from_numpy(x).cuda()
    raw = torch.zeros((300, 40), dtype=torch.float32, device="cuda")
    bad = GpuGuide(acc, seed=4, fault_injection=1)
    with pytest.raises(SpgpuError, match="timed out") as e:
        bad.mlp(feat, raw)
    assert "(-6)" in str(e.value)   # SPGPU_EKERNEL
    # the same context, a fresh guiding state: the network runs and matches the oracle
    good = GpuGuide(acc, seed=4)
    good.mlp(feat, raw)
    torch.cuda.synchronize()
    ref, _ = go.forward(good.params(), x, emulate_bf16=True)
    got = raw.cpu().numpy()
    assert np.abs(got - ref).max() <= 2e-2 * np.abs(ref).max()
    # and the context still renders
    from spica_gb300 import GpuPathIntegrator
    f = GpuPathIntegrator(seed=1).render(acc.scene.camera, acc, {"width": 8, "height": 8, "maxDepth": 4,
                                                                 "sampleCount": 4})
    assert np.all(f[..., 3] == 4)
