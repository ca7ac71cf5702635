// cuda_runtime.h stand-in for the CPU emulation (tests/emu/cj_emu.h).  TEST INFRASTRUCTURE ONLY.
#pragma once
#include "../cj_emu.h"
