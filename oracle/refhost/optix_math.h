/* Stand-in for <optix_math.h>: the vector types and helpers are in rtshim.h. */
#pragma once
#include "rtshim.h"
