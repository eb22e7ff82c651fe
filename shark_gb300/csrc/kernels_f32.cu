// FP32 instantiation of the step kernels (mixed-precision path): FP32 state and flux/update,
// FP64 drag, dt and totals arithmetic.  Built with FMA contraction enabled.
#include "kernels_impl.cuh"
namespace shark {
SHARK_INSTANTIATE(float)
}
