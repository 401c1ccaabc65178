/* Stand-in for the CUDA samples' helper_functions.h (not installed). */
#pragma once
#include <cstring>
