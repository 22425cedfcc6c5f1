// Library identification for loaders and tests.
#include "common.cuh"

extern "C" int igd_version(void) { return 100; }
