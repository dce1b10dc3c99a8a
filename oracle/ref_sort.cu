// The sort step of visionaray's GPU LBVH build, for timing that build on the GPU host.
// BENCHMARK INFRASTRUCTURE ONLY (nothing in the product links it).
//
// lbvh_builder::build (detail/bvh/lbvh.h:737-755) sorts its prim refs -- {int id;
// unsigned morton_code;}, ordered by prim_ref::operator< on the code alone (lbvh.h:
// 98-110) -- with cub::DeviceMergeSort::StableSortKeys.  That call lives in host code,
// which the cubin of oracle/ref_gpu.cu cannot carry, so it is made here against the
// CUDA toolkit's own CUB headers (library code, present on every machine): the same
// record layout, the same comparison, the same CUB algorithm.  Built by oracle/build.py
// into oracle/_build/libref_sort.so wherever nvcc is.

#include <cstddef>
#include <cstdint>

#include <cub/device/device_merge_sort.cuh>

namespace {

struct prim_ref_rec
{
    int id;
    unsigned morton_code;
};
static_assert(sizeof(prim_ref_rec) == 8, "prim ref layout");

struct code_less
{
    __device__ bool operator()(prim_ref_rec const& a, prim_ref_rec const& b) const
    {
        return a.morton_code < b.morton_code;
    }
};

} // namespace

// Temporary storage StableSortKeys wants for n records (0 on a CUDA error).
extern "C" size_t vsnray_ref_sort_bytes(uint32_t n)
{
    size_t bytes = 0;
    if (cub::DeviceMergeSort::StableSortKeys(nullptr, bytes, static_cast<prim_ref_rec*>(nullptr), int64_t(n),
                                             code_less()) != cudaSuccess)
        return 0;
    return bytes;
}

// Sorts n records in place on `stream`; returns the cudaError_t of the call.
extern "C" int vsnray_ref_sort(void* temp, size_t temp_bytes, void* records, uint32_t n, void* stream)
{
    size_t bytes = temp_bytes;
    return int(cub::DeviceMergeSort::StableSortKeys(temp, bytes, static_cast<prim_ref_rec*>(records), int64_t(n),
                                                    code_less(), static_cast<cudaStream_t>(stream)));
}
