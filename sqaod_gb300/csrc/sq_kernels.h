// sq_kernels.h -- internal declarations shared by the CUDA translation units.
#pragma once

#include "../../include/sqaod_gb300.h"
