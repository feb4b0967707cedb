// Stand-in for the CUDA samples' helper_functions.h (only <cassert> is used).
#pragma once
#include <cassert>
