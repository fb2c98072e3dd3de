"""rast_backward_mse: the mean-squared-error loss's gradient image,
(canvas - target) * scale, formed inside the backward's pixel kernel, against
rast_backward fed the same image computed by torch.  Both round the
difference and the product alike, so the per-pixel values agree bit for bit
and the gradients differ only by the order of the FP32 atomic sums."""
import numpy as np
import pytest
import torch

from jaxrenderer_gb300 import _lib
from jaxrenderer_gb300 import batch as jb
from jaxrenderer_gb300 import synthetic

pytestmark = pytest.mark.gpu

F32 = np.float32


def _assert_grads_close(got, want):
    for k in want:
        # only the order of the FP32 atomic sums differs between the two calls
        # (the per-scene terms add ~1e4 contributions of either sign): atol
        # 1e-6 of the tensor's largest entry, as for the tiled-vs-plain check
        atol = max(1e-5, 1e-6 * float(want[k].abs().max()))
        torch.testing.assert_close(got[k], want[k], rtol=1e-4, atol=atol, msg=k)


@pytest.mark.parametrize("form,layers", [("tiled", 0), ("plain", 0), ("tiled", 3)])
def test_mse_backward_matches_gradient_image(cuda_device, form, layers):
    n = 12
    inst = synthetic.brax_like_instances(n, seed=synthetic.BASE_SEED + 61)
    sb, _ = jb.scene_batch_from_instances(inst, 84, 84, shadow_size=(128, 128), device=cuda_device)
    if layers:
        opacity = np.linspace(0.3, 0.8, n).astype(F32)
        jb.set_layers(sb, layers, _lib.MIX_OVER, opacity=opacity, background=(0.2, 0.4, 0.6))
    r = jb.BatchRunner(sb, form=form)
    r.run()
    gen = torch.Generator().manual_seed(7)
    target = torch.rand(r.canvas.shape, generator=gen).to(cuda_device)
    scale = 2.0 / target.numel()
    want = {k: v.clone() for k, v in r.backward((r.canvas - target) * scale).items()}
    got = {k: v.clone() for k, v in r.backward_mse(target).items()}  # default scale: 2 / n
    # accumulate: two calls into the same arrays add up
    acc = r.grad_buffers()
    r.backward_mse(target, scale, out=acc, accumulate=True)
    r.backward_mse(target, scale, out=acc, accumulate=True)
    torch.cuda.synchronize()
    _assert_grads_close(got, want)
    _assert_grads_close({k: v * 0.5 for k, v in acc.items()}, want)
    assert want["position"].abs().sum() > 0
    assert want["job_params"].abs().sum() > 0


def test_mse_backward_refuses_a_mismatched_target(cuda_device):
    inst = synthetic.brax_like_instances(2, seed=synthetic.BASE_SEED + 62)
    sb, _ = jb.scene_batch_from_instances(inst, 32, 32, device=cuda_device)
    r = jb.BatchRunner(sb, form="tiled")
    r.run()
    with pytest.raises(ValueError, match="target shape"):
        r.backward_mse(torch.zeros((2, 32, 31, 3), device=cuda_device))
