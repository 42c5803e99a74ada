/* Test infrastructure: the reference's own libigl marching cubes (vendored in its
 * include/igl/copyleft/), found next on the include path; see ../ref_dyn.h for the rest. */
#pragma once
#include "../ref_dyn.h"
#include_next <igl/copyleft/marching_cubes.h>
