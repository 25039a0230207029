// data.h -- MOD_kernels/updates.cu:6 includes "data.h"; the header is Data.h
// (a case-insensitive file system finds it).  TEST INFRASTRUCTURE.
#include "Data.h"
