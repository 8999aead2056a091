"""Engine flag bits.

Bits 2..9 are the reference's ``mds::Flags`` (src/flags.h:6-14); the CUDA
engine honours FLOAT, OPENCL (routed here) and LEFT_TRUNCATION and accepts the
CPU-only bits (TBB, SSE, AVX, AVX512) without effect. Bits 10.. are this
engine's own.
"""
FLOAT = 1 << 2
TBB = 1 << 3
OPENCL = 1 << 4
LEFT_TRUNCATION = 1 << 5
SSE = 1 << 7
AVX = 1 << 8
AVX512 = 1 << 9
CUDA = 1 << 10
DELTA_F32 = 1 << 11
DOUBLE_FLOAT = 1 << 12  # FP64-accurate double-float pair math on the FP32 pipes (P <= 6)

MAX_DIMENSION = 10

# Sweep schedules (include/mdsx.h MDSX_SWEEP_*).
SWEEP_ROWS = 0
SWEEP_PAIRS = 1
