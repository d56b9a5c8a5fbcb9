"""The reference's kernel launch functions (cuda_ray_tracer/kernels/RayCastKernel.hpp:47-74) over the C ABI.

Same names, argument meaning and semantics: every call is synchronous (the reference synchronises the
device after each launch, RayCastKernel.cu:831-832). The two texture objects of the reference's
RayCastKernelInput are replaced by one resident :class:`~phantasyenginetestbed_gb300.Scene`; rays and
results are device buffers (torch CUDA tensors or raw addresses). Errors raise PheError instead of
being printed and ignored.
"""
from __future__ import annotations

from dataclasses import dataclass

from . import Scene, cast_any, cast_closest, cast_closest_plain, gen_primary_rays
from .native import CameraDef


@dataclass
class RayCastKernelInput:
    """RayCastKernel.hpp:50-55: bvhNodes + triangleVerts (here one Scene), numRays, rays."""
    scene: Scene
    numRays: int
    rays: object


def _sync():
    import torch
    torch.cuda.synchronize()


def launchRayCastKernel(input: RayCastKernelInput, rayResults, deviceProperties=None) -> None:
    """Closest hit, persistent kernel (RayCastKernel.cu:806-839)."""
    cast_closest(input.scene, input.rays, rayResults, input.numRays)
    _sync()


def launchRayCastNoPersistenceKernel(input: RayCastKernelInput, rayResults, deviceProperties=None) -> None:
    """Closest hit, one ray per thread (RayCastKernel.cu:841-851)."""
    cast_closest_plain(input.scene, input.rays, rayResults, input.numRays)
    _sync()


def launchShadowRayCastKernel(input: RayCastKernelInput, inLight, deviceProperties=None) -> None:
    """Any hit: inLight[i] = 1 when nothing lies in [tMin, tMax) (RayCastKernel.cu:853-886)."""
    cast_any(input.scene, input.rays, inLight, input.numRays)
    _sync()


def launchGenPrimaryRaysKernel(rays, cam: CameraDef, res) -> None:
    """Primary rays in 8x8-tile order (RayCastKernel.cu:899-919, 971-982)."""
    order = 1 if res[0] % 8 == 0 and res[1] % 8 == 0 else 0
    gen_primary_rays(rays, cam, res, order=order)
    _sync()
