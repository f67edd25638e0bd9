// Host-side (CPU-only) parts of the fggpu library: mesh ingest and set-up, settings,
// output files and the time-integration driver. Declared in include/fggpu.h.
#pragma once

#include "../../include/fggpu.h"
