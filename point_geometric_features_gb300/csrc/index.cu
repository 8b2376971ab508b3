// index.cu -- resident grid index (pgeof_index_*): one cloud's grid built once
// and then searched any number of times, with any k or radius, for the cloud's
// own points or for external queries, and fed to the fused kNN -> feature
// pipeline. The reference rebuilds its nanoflann KD-tree inside every call
// (include/nn_search.hpp:35,39,90,97; include/pgeof.hpp:330,333); results here
// are the per-call entry points' results exactly, since the search is exact
// for any cell size.
//
// Lifetime and streams: pgeof_index_create_f32 builds on the caller's stream
// and synchronises it, so the index is complete and immutable when it returns
// and any stream of the same device may search it concurrently. Every search
// records an event on its stream; pgeof_index_destroy makes the index's own
// stream wait for those events before the memory goes back to the pool.
#include <mutex>
#include <utility>
#include <vector>

#include "kernels.cuh"

namespace pgeof {
namespace {

// xyz4[p.idx] = p for every point of the cell-ordered copy: the padded
// original-order coordinates the feature kernels gather from.
__global__ void cell_points_to_xyz4_kernel(const SPoint<float>* __restrict__ pts, uint64_t n,
                                           float4* __restrict__ xyz4) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const SPoint<float> p = pts[i];
        xyz4[p.idx] = make_float4(p.x, p.y, p.z, 0.0f);
    }
}

struct ResidentIndex {
    int device = -1;
    uint64_t n = 0;
    uint32_t k_hint = 0;
    float radius_hint = 0.0f;
    GridIndex<float> grid;
    Scratch xyz4;
    cudaStream_t own = nullptr;
    std::mutex mu;
    std::vector<std::pair<cudaStream_t, cudaEvent_t>> uses;

    ~ResidentIndex() {
        if (own) {
            for (auto& u : uses) cudaStreamWaitEvent(own, u.second, 0);
            // frees are enqueued on `own`, after every recorded use
            grid.cell_mem.s = own;
            grid.pts_mem.s = own;
            xyz4.s = own;
        }
        grid.cell_mem.reset();
        grid.pts_mem.reset();
        xyz4.reset();
        if (own) {
            cudaStreamSynchronize(own);
            cudaStreamDestroy(own);
        }
        for (auto& u : uses) cudaEventDestroy(u.second);
    }

    // Marks the work just enqueued on `s` as a use of the index.
    int record_use(cudaStream_t s) {
        std::lock_guard<std::mutex> lk(mu);
        cudaEvent_t ev = nullptr;
        for (auto& u : uses)
            if (u.first == s) ev = u.second;
        if (!ev) {
            PGEOF_CUDA_TRY(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            uses.emplace_back(s, ev);
        }
        PGEOF_CUDA_TRY(cudaEventRecord(ev, s));
        return PGEOF_OK;
    }
};

int resolve(pgeof_index handle, ResidentIndex** out) {
    ResidentIndex* ix = reinterpret_cast<ResidentIndex*>(handle);
    if (!ix) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid index");
    int dev = -1;
    PGEOF_CUDA_TRY(cudaGetDevice(&dev));
    if (dev != ix->device)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "the index lives on device " + std::to_string(ix->device) +
                                                    ", the current device is " + std::to_string(dev));
    *out = ix;
    return PGEOF_OK;
}

int check_queries(const float* query, int64_t n_query) {
    if (n_query < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "query has a negative size");
    if ((uint64_t)n_query > 0xfffffffeull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "query exceeds 2^32-2 points");
    return PGEOF_OK;  // (query == NULL: the indexed points, n_query ignored)
}

// Queries in the grid's cell order: the indexed points themselves (query ==
// NULL; rows come out in the cloud's original order) or `query` sorted.
int cell_queries(const ResidentIndex& ix, const float* query, int64_t n_query, Scratch& qmem, Scratch& qstart,
                 const SPoint<float>** q, uint64_t* m, cudaStream_t s) {
    if (!query) {
        *q = ix.grid.pts;
        *m = ix.n;
        return PGEOF_OK;
    }
    SPoint<float>* sorted = nullptr;
    PGEOF_TRY(sort_queries<float>(query, (uint64_t)n_query, ix.grid.g, qmem, &sorted, qstart, s));
    *q = sorted;
    *m = (uint64_t)n_query;
    return PGEOF_OK;
}

}  // namespace
}  // namespace pgeof

using namespace pgeof;

extern "C" {

int pgeof_index_create_f32(const float* data, int64_t n_data, uint32_t k_hint, float radius_hint,
                           pgeof_stream_t stream, pgeof_index* out) {
    if (!out) return fail(PGEOF_ERR_INVALID_ARGUMENT, "out is NULL");
    *out = nullptr;
    if (n_data < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "the index needs at least one point");
    if ((uint64_t)n_data > 0xfffffffeull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "data exceeds 2^32-2 points");
    if (!data) return fail(PGEOF_ERR_INVALID_ARGUMENT, "data is NULL");
    if (!(radius_hint >= 0.0f)) return fail(PGEOF_ERR_INVALID_ARGUMENT, "radius_hint must be >= 0");
    const cudaStream_t s = (cudaStream_t)stream;
    ResidentIndex* ix = new ResidentIndex();
    ix->n = (uint64_t)n_data;
    ix->k_hint = k_hint ? k_hint : 16u;
    ix->radius_hint = radius_hint;
    int st = PGEOF_OK;
    if (cudaGetDevice(&ix->device) != cudaSuccess) st = fail(PGEOF_ERR_CUDA, "cudaGetDevice");
    // the cell-size rule of the per-call entry points: kNN steers the occupancy
    // towards k, a radius clamps the edge to [r/4, r]
    if (st == PGEOF_OK)
        st = build_grid<float>(data, ix->n, ix->k_hint, radius_hint / 4.0f, radius_hint, ix->grid, s);
    if (st == PGEOF_OK) st = ix->xyz4.alloc(ix->n * sizeof(float4), s);
    if (st == PGEOF_OK) {
        const int blocks = (int)std::min<uint64_t>((ix->n + 255) / 256, 4096);
        KernelTimer kt("cell_points_to_xyz4_kernel", s);
        cell_points_to_xyz4_kernel<<<blocks, 256, 0, s>>>(ix->grid.pts, ix->n, ix->xyz4.as<float4>());
        count_launch();
        st = check_launch("cell_points_to_xyz4_kernel");
    }
    if (st == PGEOF_OK && cudaStreamSynchronize(s) != cudaSuccess) st = fail(PGEOF_ERR_CUDA, "index build");
    if (st == PGEOF_OK && cudaStreamCreateWithFlags(&ix->own, cudaStreamNonBlocking) != cudaSuccess)
        st = fail(PGEOF_ERR_CUDA, "cudaStreamCreateWithFlags");
    if (st != PGEOF_OK) {
        delete ix;
        return st;
    }
    *out = reinterpret_cast<pgeof_index>(ix);
    return PGEOF_OK;
}

int pgeof_index_destroy(pgeof_index index) {
    delete reinterpret_cast<ResidentIndex*>(index);
    return PGEOF_OK;
}

int pgeof_index_size(pgeof_index index, int64_t* n_points) {
    ResidentIndex* ix = reinterpret_cast<ResidentIndex*>(index);
    if (!ix || !n_points) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid index or NULL output");
    *n_points = (int64_t)ix->n;
    return PGEOF_OK;
}

int pgeof_index_knn_search_f32(pgeof_index index, const float* query, int64_t n_query, uint32_t knn,
                               uint32_t* indices, float* sqr_dist, pgeof_stream_t stream) {
    ResidentIndex* ix = nullptr;
    PGEOF_TRY(resolve(index, &ix));
    PGEOF_TRY(check_queries(query, n_query));
    if ((uint64_t)knn > ix->n)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size");
    if ((query && n_query == 0) || knn == 0) return PGEOF_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    Scratch qmem, qstart;
    const SPoint<float>* q = nullptr;
    uint64_t m = 0;
    PGEOF_TRY(cell_queries(*ix, query, n_query, qmem, qstart, &q, &m, s));
    SearchOut<float> o;
    o.indices = indices;
    o.sqr_dist = sqr_dist;
    const int st = launch_search<float>(ix->grid, q, nullptr, m, MODE_KNN, knn, 0.0f, o, s);
    PGEOF_TRY(ix->record_use(s));
    return st;
}

int pgeof_index_radius_search_f32(pgeof_index index, const float* query, int64_t n_query, float search_radius,
                                  uint32_t max_knn, int32_t* indices, float* sqr_dist, pgeof_stream_t stream) {
    ResidentIndex* ix = nullptr;
    PGEOF_TRY(resolve(index, &ix));
    PGEOF_TRY(check_queries(query, n_query));
    if ((uint64_t)max_knn > ix->n)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "max knn size is greater than the data point cloud size");
    if ((query && n_query == 0) || max_knn == 0) return PGEOF_OK;
    const cudaStream_t s = (cudaStream_t)stream;
    Scratch qmem, qstart;
    const SPoint<float>* q = nullptr;
    uint64_t m = 0;
    PGEOF_TRY(cell_queries(*ix, query, n_query, qmem, qstart, &q, &m, s));
    SearchOut<float> o;
    o.indices = indices;
    o.sqr_dist = sqr_dist;
    o.radius_fill_last = true;
    const int st = launch_search<float>(ix->grid, q, nullptr, m, MODE_RADIUS, max_knn, search_radius, o, s);
    PGEOF_TRY(ix->record_use(s));
    return st;
}

int pgeof_index_knn_features_f32(pgeof_index index, uint32_t knn, const uint32_t* k_scales, int64_t n_scales,
                                 float* features, pgeof_stream_t stream) {
    ResidentIndex* ix = nullptr;
    PGEOF_TRY(resolve(index, &ix));
    if (knn == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn should be >= 1");
    if ((uint64_t)knn > ix->n)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size");
    if (n_scales < 0 || (n_scales > 0 && !k_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    for (int64_t i = 0; i < n_scales; ++i)  // the rule of check_scales, include/pgeof.hpp:123-133
        if (k_scales[i] < (i > 0 ? k_scales[i - 1] : 1u))
            return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    if (n_scales > 0 && k_scales[n_scales - 1] > knn)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales must not exceed knn");
    const cudaStream_t s = (cudaStream_t)stream;
    // neighbour rows in cell order, no distances; the feature pass walks them in
    // that order and writes each row to its original position
    Scratch nn;
    PGEOF_TRY(nn.alloc((size_t)ix->n * knn * sizeof(uint32_t), s));
    SearchOut<float> o;
    o.indices = nn.p;
    o.sqr_dist = nullptr;
    o.rows_in_query_order = true;
    int st = launch_search<float>(ix->grid, ix->grid.pts, nullptr, ix->n, MODE_KNN, knn, 0.0f, o, s);
    if (st == PGEOF_OK)
        st = launch_features(ix->xyz4.as<float4>(), ix->n, nn.as<uint32_t>(), ix->n * knn, nullptr, ix->n,
                             n_scales == 0, 1, k_scales, (int)n_scales, features, nullptr, s, nullptr, 0,
                             ix->grid.pts, knn);
    PGEOF_TRY(ix->record_use(s));
    return st;
}

}  // extern "C"
