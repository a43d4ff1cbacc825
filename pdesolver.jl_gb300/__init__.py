"""GB300-native Euler SBP hot path: host-side set-up (operators, meshes) and
the ctypes mirror of the C-ABI library ``libeulergpu.so``."""
