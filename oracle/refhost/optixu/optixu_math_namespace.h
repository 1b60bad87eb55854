/* Stand-in for <optixu/optixu_math_namespace.h>: see rtshim.h. */
#pragma once
#include "../rtshim.h"
