"""The launch-shape autotuner of the 32-slot E passes (cpm_opset_autotune):
it picks shapes from its candidate lists, keeps them with the operator, and
no shape changes a result (the FP32 and FP64 32-slot applies give the same
bits before tuning, after it, and with hand-set extreme shapes)."""
import pytest

from test_gpu_setup import two_circle_ibcs

pytestmark = pytest.mark.gpu


def _applies(gpu, O, x32, x64):
    import torch

    out = []
    for x, fp32 in ((x32, True), (x64, False)):
        t, y = torch.empty_like(x), torch.empty_like(x)
        O.apply_device(0.0, -1.0, 32, fp32, x.data_ptr(), t.data_ptr(), y.data_ptr())
        gpu.sync()
        out += [t.clone(), y.clone()]
    return out


def test_autotune_choices_and_results_unchanged(gpu):
    import torch

    dx = 0.05
    O = gpu.OpSet(gpu.Tube(gpu.desc(gpu.SPHERE, [1.0]), 3, dx), two_circle_ibcs(gpu, dx))
    gen = torch.Generator().manual_seed(3)
    x32 = (torch.rand((O.D, 32), generator=gen, dtype=torch.float32) * 2 - 1).cuda()
    x64 = (torch.rand((O.D, 32), generator=gen, dtype=torch.float64) * 2 - 1).cuda()
    ref = _applies(gpu, O, x32, x64)
    r = O.autotune(reps=5, fp64=True)
    assert r["e32_blocks_per_sm"] in (8, 16, 24, 32, 48, 64, 96, 128)
    assert r["patch_blocks_per_sm"] in (4, 8, 16, 32, 64, 128)
    assert r["e64_blocks_per_sm"] in (4, 8, 16, 32, 64)
    assert 0 < r["e32_us"] <= r["e32_default_us"] and 0 < r["patch_us"] <= r["patch_default_us"]
    assert 0 < r["e64_us"] <= r["e64_default_us"]
    for a, b in zip(ref, _applies(gpu, O, x32, x64)):
        assert torch.equal(a, b)
    O.set_launch(1, 1, 1)
    for a, b in zip(ref, _applies(gpu, O, x32, x64)):
        assert torch.equal(a, b)
    O.set_launch(1024, 1024, 1024)
    for a, b in zip(ref, _applies(gpu, O, x32, x64)):
        assert torch.equal(a, b)
    with pytest.raises(gpu.CpmError):
        O.set_launch(-1, 0, 0)
