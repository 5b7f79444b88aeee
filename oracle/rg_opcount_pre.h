// Forced first include of the op-counting build of the oracle (rg_opcount.cpp
// and the Makefile's opcount target) -- MEASUREMENT INFRASTRUCTURE ONLY.
// The standard headers the oracle uses are included here, before `double`
// is redefined, so that only the oracle's own text sees the counting type.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "rg_opcount.h"

#define RG_OPCOUNT 1
#define double rg_count::Real
