/* Stand-in for <optix_world.h>: everything the reference's programs use is in rtshim.h. */
#pragma once
#include "rtshim.h"
