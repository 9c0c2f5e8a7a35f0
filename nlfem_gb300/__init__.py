"""GB300-native nonlocal finite-element assembly (drop-in for nlfem's assembly path).

Public surface: ``nlfem_gb300.nlfem`` mirrors the reference's Python module; the C ABI is
declared in include/nlfem_gpu.h and implemented in libnlfem_gpu.so (built by ``build.build``).
"""
__all__ = ["nlfem", "meshes", "quadrules", "build"]
