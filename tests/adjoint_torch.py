"""torch.autograd.Function over rdc_forward / rdc_backward (test harness only).

Parameters are per-object tensors: albedo (N, 3), roughness (N), emission
(N, 3, the emitted radiance emission_color * emission_strength).  Forward
writes them into a copy of the scene (emission as colour with strength 1,
which gives the same product) and renders the mean-radiance image."""
import copy

import numpy as np
import torch

from raydar_gb300 import CudaRenderer


def scene_with(scene, albedo, roughness, emission):
    s = copy.deepcopy(scene)
    for j, o in enumerate(s.objects):
        o.material.albedo = np.asarray(albedo[j], np.float32).copy()
        o.material.roughness = float(np.float32(roughness[j]))
        o.material.emission_color = np.asarray(emission[j], np.float32).copy()
        o.material.emission_strength = 1.0
    return s


class RenderFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, albedo, roughness, emission, renderer: CudaRenderer, scene, spp: int):
        s = scene_with(scene, albedo.detach().cpu().numpy(), roughness.detach().cpu().numpy(),
                       emission.detach().cpu().numpy())
        img = renderer.forward(s, spp)
        ctx.renderer = renderer
        ctx.scene = s
        return torch.from_numpy(img.copy())

    @staticmethod
    def backward(ctx, grad_image):
        ga, gr, ge = ctx.renderer.backward(ctx.scene, grad_image.detach().cpu().numpy())
        return torch.from_numpy(ga), torch.from_numpy(gr), torch.from_numpy(ge), None, None, None


def material_tensors(scene):
    albedo = torch.tensor(np.stack([o.material.albedo for o in scene.objects]), dtype=torch.float32)
    roughness = torch.tensor([o.material.roughness for o in scene.objects], dtype=torch.float32)
    emission = torch.tensor(np.stack([np.asarray(o.material.emission_color, np.float32) *
                                      np.float32(o.material.emission_strength) for o in scene.objects]),
                            dtype=torch.float32)
    return albedo, roughness, emission
