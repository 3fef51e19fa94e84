// Kernel table of the test suite's Brusselator model, double-word sweeps
// included (include/va_model.cuh): its own nvcc unit and shared library.
#include "va_model.cuh"

#include "user_models.cuh"

VA_DEFINE_MODEL_DW(Brusselator, brusselator_kernels)
