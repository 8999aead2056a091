// Test scaffolding: forwards to the std::thread TBB stand-in (see tbb_shim_common.h).
#pragma once
#include "tbb_shim_common.h"
