// Instantiations of the block Fock-build kernels (jk_blocks.cuh), kept out of
// eri.cu so that they compile in parallel with it.
#include "jk_blocks.cuh"

namespace hfgpu {

DigestFn digest_fn(int tb, int tk)
{
#define HF_D(B, K) \
    if (tb == B && tk == K) return digest_kernel<B, K>;
    HF_D(0, 0) HF_D(0, 1) HF_D(0, 2) HF_D(0, 3) HF_D(0, 4) HF_D(0, 5)
    HF_D(1, 1) HF_D(1, 2) HF_D(1, 3) HF_D(1, 4) HF_D(1, 5)
    HF_D(2, 2) HF_D(2, 3) HF_D(2, 4) HF_D(2, 5)
    HF_D(3, 3) HF_D(3, 4) HF_D(3, 5)
    HF_D(4, 4) HF_D(4, 5)
    HF_D(5, 5)
#undef HF_D
    return nullptr;
}

DigestFn digest_wide_fn(int tb, int tk)
{
#define HF_D(B, K) \
    if (tb == B && tk == K) return digest_wide_kernel<B, K>;
    HF_D(0, 0) HF_D(0, 1) HF_D(0, 2) HF_D(0, 3) HF_D(0, 4) HF_D(0, 5)
    HF_D(1, 1) HF_D(1, 2) HF_D(1, 3) HF_D(1, 4) HF_D(1, 5)
    HF_D(2, 2) HF_D(2, 3) HF_D(2, 4) HF_D(2, 5)
    HF_D(3, 3) HF_D(3, 4) HF_D(3, 5)
    HF_D(4, 4) HF_D(4, 5)
    HF_D(5, 5)
#undef HF_D
    return nullptr;
}

}  // namespace hfgpu
