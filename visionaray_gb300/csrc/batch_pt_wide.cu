// The batched path tracer over the arena's 4- and 8-wide nodes (batch_pt.cuh); in its
// own translation unit so that it compiles in parallel with the node-pair kernels.
// Compiled with --fmad=false like batch_pt.cu.

#include "batch_pt.cuh"

namespace gbrt {
namespace {

template <int Width, bool Extended, bool Lit>
batch_kernel pick_block_wide(uint32_t block)
{
    // the pair stack's size is unused by the wide kernels (their own stack): 16
    switch (block)
    {
    case 128: return batch_pt<128, 16, Extended, Lit, Width>;
    case 256: return batch_pt<256, 16, Extended, Lit, Width>;
    case 512: return batch_pt<512, 16, Extended, Lit, Width>;
    default: return nullptr;
    }
}

template <int Width>
batch_kernel pick_width(gbrt_batch_launch const& l, bool extended, bool lit)
{
    if (lit) return extended ? pick_block_wide<Width, true, true>(l.block) : pick_block_wide<Width, false, true>(l.block);
    return extended ? pick_block_wide<Width, true, false>(l.block) : pick_block_wide<Width, false, false>(l.block);
}

} // namespace

batch_kernel pick_wide_kernel(gbrt_batch_launch const& l, bool extended, bool lit)
{
    if (l.width == 4) return pick_width<4>(l, extended, lit);
    if (l.width == 8) return pick_width<8>(l, extended, lit);
    return nullptr;
}

} // namespace gbrt
