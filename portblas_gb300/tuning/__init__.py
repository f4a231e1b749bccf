"""Autotuner sweep, MLP training and regret evaluation of the FP32 GEMM tile
selector (see portblas_gb300/csrc/selector.cu for the configuration space)."""
