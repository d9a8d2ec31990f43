"""GB300-native RPA response path of 2DMaterialsOpticalProps.

Package contents:
  csrc/      CUDA kernels and the C ABI (include/rpa_gpu.h) -> librpa_gb300.so
  build.py   in-tree nvcc build for sm_103a
  rpa.py     ctypes binding of the C ABI (the drivers' call sequence)
  synth.py   seeded synthetic Bloch bases in the drivers' array layouts
"""
