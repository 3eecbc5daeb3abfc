"""Scene ingestion into the flattened scene the C ABI uploads
(crates/pyre/src/io): PBRT subset, glTF 2.0 meshes, Radiance .hdr maps."""
from .gltf import GltfError, load_gltf
from .hdr import HdrLoadError, load_hdri
from .pbrt import LoadedPbrt, PbrtError, load_pbrt

__all__ = ["GltfError", "HdrLoadError", "LoadedPbrt", "PbrtError", "load_gltf", "load_hdri", "load_pbrt"]
