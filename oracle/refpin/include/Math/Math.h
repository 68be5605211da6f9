// Stand-in for OpenEngine's Math/Math.h (nothing of it is used by the pinned
// functions).  TEST INFRASTRUCTURE ONLY.
#pragma once
