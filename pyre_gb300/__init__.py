"""GB300 (sm_103a) wavefront path tracer for the Pyre renderer's hot path.

The compute path is libpyre_cuda.so (hand-written CUDA kernels behind a C ABI,
include/pyre_cuda.h); this package holds its ctypes binding, a host-side
mirror of the reference's scene API and the scene presets.
"""
from .scene import (CameraSpec, CudaIntegrator, DeviceScene, DiffuseAreaQuadLight, DisneyBsdf, Film,  # noqa: F401
                    HdriEnvironmentLight, InstanceMotion, Lambertian, MeshInstance, PathIntegrator, PinholeCamera,
                    Primitive, Scene, ThinLensCamera, TriangleMesh, build_bvh, pixel_seed)

__all__ = ["CameraSpec", "CudaIntegrator", "DeviceScene", "DiffuseAreaQuadLight", "DisneyBsdf", "Film",
           "HdriEnvironmentLight", "InstanceMotion", "Lambertian", "MeshInstance", "PathIntegrator", "PinholeCamera",
           "Primitive", "Scene", "ThinLensCamera", "TriangleMesh", "build_bvh", "pixel_seed"]
