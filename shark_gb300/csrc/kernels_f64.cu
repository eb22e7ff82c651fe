// FP64 instantiation of the step kernels.  Built with --fmad=false so that every operation
// rounds exactly like the CPU oracle (which is built with -ffp-contract=off).
#include "kernels_impl.cuh"
namespace shark {
SHARK_INSTANTIATE(double)
}
