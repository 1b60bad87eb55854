/* Stand-in for the OptiX 6.0 SDK header <optix.h> (not in the reference's
 * tree).  Test infrastructure: see rtshim.h. */
#pragma once
#include "rtshim.h"
