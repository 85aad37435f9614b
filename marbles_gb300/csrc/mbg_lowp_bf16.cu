// mbg_lowp_bf16.cu -- the 16-bit form's kernels for BF16 storage (a translation unit of its
// own so that the two formats compile in parallel).
#include "mbg_lowp_kern.cuh"

namespace mbg {
template struct Lowp16<true>;
}  // namespace mbg
