/* Test infrastructure: libigl stand-in (declarations only); see ref_dyn.h. */
#pragma once
#include "ref_dyn.h"
