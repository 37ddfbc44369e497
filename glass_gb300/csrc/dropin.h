// Shared by the drop-in entry points: the calling thread's GPU context (one
// per host thread, created on first use on device $GLASS_GPU_DEVICE or 0), and
// the reference's way of failing (message on stderr, exit).
#pragma once
#include "../../include/glass_gb300.h"

glass_gpu_ctx *dropin_ctx(const char *who);
[[noreturn]] void dropin_fail(const char *who);
