"""voxplat_gb300 — GB300-native (sm_103a) voxel geometry pipeline.

The product is the C-ABI library libvoxgpu.so (include/voxgpu.h). This
package builds it in-tree and binds it with ctypes (`voxplat_gb300.gpu`);
there is no CPU fallback: if the library cannot be loaded, every GPU entry
point raises.
"""
__all__ = ["build", "gpu", "worldgen"]
