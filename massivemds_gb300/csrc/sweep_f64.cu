// Sweep kernel instances: FP64 pair arithmetic over FP64-stored delta (P = 1..10, truncation on/off).
#include "sweep_dispatch.cuh"

MDSX_DEFINE_MODE(f64, double, double)
