// sq_kernels.h -- internal declarations shared by the CUDA translation units.
#pragma once

#include "../../include/sqaod_gb300.h"

// sets the message returned by sq103_last_error() on this thread
void sq103_set_error(const char *msg);
