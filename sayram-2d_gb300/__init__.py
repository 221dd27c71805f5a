"""GB300-native Sayram-2D hot path: PPFV assembly + implicit solve on one GPU.

The compute lives in the CUDA shared library built from ``csrc/`` (C-ABI in
``include/sayram_gpu.h``); this package holds the Python-side binding of that C-ABI, the case
generators and the build helper.
"""
