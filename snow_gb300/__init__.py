"""GB300-native explicit snow-MPM step (sm_103a CUDA kernels behind a C ABI)."""
