// Kernel table of the test suite's forced Duffing model, built the way a user
// of the library builds one (include/va_model.cuh): its own nvcc unit and
// shared library, -fmad=false.
#include "va_model.cuh"

#include "user_models.cuh"

VA_DEFINE_MODEL(ForcedDuffing, forced_duffing_kernels)
