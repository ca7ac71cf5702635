#pragma once
#include "cj_thrust_emu.h"
