// Stand-in for extensions-CUDA's logger extensions (stream operators for the
// CUDA vector types; the observer logger of Meta/CUDA.h takes them itself).
// TEST INFRASTRUCTURE ONLY.
#pragma once
#include <Meta/CUDA.h>
