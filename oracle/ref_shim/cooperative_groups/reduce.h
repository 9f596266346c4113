/* Compile-only stand-in (see ../cooperative_groups.h). */
#pragma once
#include "../cooperative_groups.h"
