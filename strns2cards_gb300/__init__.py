"""GB300-native strands-to-cards rasterization path (sm_103a CUDA behind a C ABI)."""
