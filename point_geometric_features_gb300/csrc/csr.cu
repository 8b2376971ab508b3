// csr.cu -- radius-search table -> CSR neighbourhoods on the device.
//
// pgeof's README (README.md:157-163) turns radius_search's padded (n, max_knn)
// table into the CSR pair that compute_features* take with a host-side mask
// and cumulative sum. Here the search's own per-query counts are clamped to
// max_knn, scanned into nn_ptr, and each row's leading entries are copied to
// nn[nn_ptr[i] ..] by one warp per row (coalesced reads and writes), so the
// neighbourhoods never leave the GPU.
#include "kernels.cuh"

namespace pgeof {

namespace {

__global__ void clamp_counts_kernel(const uint32_t* __restrict__ found, uint64_t m, uint32_t max_knn,
                                    uint32_t* __restrict__ counts) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < m; i += (uint64_t)gridDim.x * blockDim.x)
        counts[i] = min(found[i], max_knn);
}

__global__ void compact_rows_kernel(const int32_t* __restrict__ table, uint64_t m, uint32_t max_knn,
                                    const uint32_t* __restrict__ nn_ptr, uint32_t* __restrict__ nn) {
    const int lane = threadIdx.x & 31;
    const uint64_t warps = (uint64_t)gridDim.x * (blockDim.x >> 5);
    for (uint64_t i = blockIdx.x * (uint64_t)(blockDim.x >> 5) + (threadIdx.x >> 5); i < m; i += warps) {
        const uint32_t b = nn_ptr[i], c = nn_ptr[i + 1] - b;
        const int32_t* row = table + i * max_knn;
        for (uint32_t j = lane; j < c; j += 32) nn[(uint64_t)b + j] = (uint32_t)row[j];
    }
}

}  // namespace

int launch_csr_from_table(const int32_t* table, const uint32_t* found, uint64_t m, uint32_t max_knn,
                          uint32_t* counts, uint32_t* partials, uint32_t* nn_ptr, uint32_t* nn, cudaStream_t s) {
    const DeviceInfo* di;
    PGEOF_TRY(current_device_info(&di));
    const unsigned cap = (unsigned)di->sm_count * 8;
    {
        KernelTimer kt("csr_kernels", s);
        clamp_counts_kernel<<<std::min<unsigned>(ceil_div_u(m, 256), cap), 256, 0, s>>>(found, m, max_knn, counts);
        count_launch();
        PGEOF_TRY(check_launch("clamp_counts_kernel"));
    }
    PGEOF_TRY(exclusive_scan_into(counts, (uint32_t)m, nn_ptr, partials, s));
    KernelTimer kt("csr_kernels", s);
    compact_rows_kernel<<<std::min<unsigned>(ceil_div_u(m, 8), cap), 256, 0, s>>>(table, m, max_knn, nn_ptr, nn);
    count_launch();
    return check_launch("compact_rows_kernel");
}

}  // namespace pgeof
