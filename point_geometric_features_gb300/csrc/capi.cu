// capi.cu -- the extern "C" entry points of libpgeof_cuda (include/pgeof_cuda.h):
// argument checks with the reference's error conditions, per-device state
// (memory pool, data-error word), the asynchronous device-pointer family and
// the synchronous host-pointer family that the Python binding uses.
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <unordered_map>
#include <string>
#include <vector>

#include "kernels.cuh"

namespace pgeof {

std::atomic<uint64_t> g_launch_count{0};
std::atomic<uint64_t> g_device_alloc_count{0};

namespace {

thread_local std::string t_last_error;
thread_local uint32_t* t_error_word_override = nullptr;
std::atomic<int> g_eig_order{0};

struct DevState {
    std::once_flag once;
    int status = PGEOF_OK;
    std::string msg;
    DeviceInfo info;
    cudaMemPool_t pool = nullptr;
    uint32_t* err_word = nullptr;
};
constexpr int kMaxDevices = 64;
DevState g_dev[kMaxDevices];

void init_device(DevState& st, int dev) {
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, dev);
    if (e != cudaSuccess) {
        st.status = PGEOF_ERR_NO_DEVICE;
        st.msg = std::string("cudaGetDeviceProperties: ") + cudaGetErrorString(e);
        return;
    }
    if (!(prop.major == 10 && prop.minor == 3)) {
        st.status = PGEOF_ERR_NO_DEVICE;
        st.msg = "libpgeof_cuda is built for sm_103a (GB300); device " + std::to_string(dev) + " is " + prop.name +
                 " (sm_" + std::to_string(prop.major) + std::to_string(prop.minor) + ")";
        return;
    }
    st.info.device = dev;
    st.info.sm_count = prop.multiProcessorCount;
    st.info.max_smem_optin = (int)prop.sharedMemPerBlockOptin;
    cudaMemPoolProps props;
    memset(&props, 0, sizeof(props));
    props.allocType = cudaMemAllocationTypePinned;
    props.handleTypes = cudaMemHandleTypeNone;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = dev;
    e = cudaMemPoolCreate(&st.pool, &props);
    if (e == cudaSuccess) {
        uint64_t keep = ~0ull;
        e = cudaMemPoolSetAttribute(st.pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    if (e == cudaSuccess) {
        e = cudaMalloc(&st.err_word, 256);
        count_device_alloc();
    }
    if (e == cudaSuccess) e = cudaMemset(st.err_word, 0, 256);
    if (e != cudaSuccess) {
        st.status = PGEOF_ERR_CUDA;
        st.msg = std::string("device initialisation: ") + cudaGetErrorString(e);
    }
}

int device_state(DevState** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        (void)cudaGetLastError();
        return fail(PGEOF_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
    }
    DevState& st = g_dev[dev];
    std::call_once(st.once, init_device, std::ref(st), dev);
    if (st.status != PGEOF_OK) return fail(st.status, st.msg);
    *out = &st;
    return PGEOF_OK;
}

cudaStream_t host_stream() {
    // one non-blocking stream per host thread and device for the host-pointer API
    thread_local cudaStream_t streams[kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (!streams[dev]) cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking);
    return streams[dev];
}

// Copy streams of the host-pointer API's feature pipeline (0: uploads, 1:
// downloads), one pair per host thread and device.
cudaStream_t host_copy_stream(int which) {
    thread_local cudaStream_t streams[2][kMaxDevices] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (!streams[which][dev]) cudaStreamCreateWithFlags(&streams[which][dev], cudaStreamNonBlocking);
    return streams[which][dev];
}

// Per-call data-error word for host-pointer calls (no cross-talk between threads).
struct CallErrors {
    Scratch word;
    cudaStream_t s;
    explicit CallErrors(cudaStream_t stream) : s(stream) {}
    int begin() {
        PGEOF_TRY(word.alloc(16, s));
        PGEOF_CUDA_TRY(cudaMemsetAsync(word.p, 0, 16, s));
        t_error_word_override = word.as<uint32_t>();
        return PGEOF_OK;
    }
    ~CallErrors() { t_error_word_override = nullptr; }
    // after the stream is synchronised
    int check() {
        uint32_t bits = 0;
        PGEOF_CUDA_TRY(cudaMemcpy(&bits, word.p, sizeof(bits), cudaMemcpyDeviceToHost));
        return bits_status(bits);
    }
    static int bits_status(uint32_t bits) {
        if (bits & ERR_NN_RANGE) return fail(PGEOF_ERR_DATA, "nn holds an index >= the number of points in xyz");
        if (bits & ERR_PTR_RANGE)
            return fail(PGEOF_ERR_DATA, "nn_ptr must be non-decreasing and its values must not exceed len(nn)");
        if (bits & ERR_INTERNAL) return fail(PGEOF_ERR_INTERNAL, "neighbour selection exceeded its refinement bound");
        return PGEOF_OK;
    }
};

template <class T>
int upload(Scratch& dst, const T* src, uint64_t count, cudaStream_t s) {
    PGEOF_TRY(dst.alloc(count * sizeof(T), s));
    if (count) PGEOF_CUDA_TRY(cudaMemcpyAsync(dst.p, src, count * sizeof(T), cudaMemcpyHostToDevice, s));
    return PGEOF_OK;
}
template <class T>
int download(T* dst, const Scratch& src, uint64_t count, cudaStream_t s) {
    if (count) PGEOF_CUDA_TRY(cudaMemcpyAsync(dst, src.p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    return PGEOF_OK;
}

int finish_host(CallErrors& ce, cudaStream_t s) {
    PGEOF_CUDA_TRY(cudaStreamSynchronize(s));
    return ce.check();
}

// ------------------------------------------------------------ validation
constexpr uint64_t kMaxPoints = 0xfffffffeull;

int check_cloud(int64_t n, const char* what) {
    if (n < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, std::string(what) + " has a negative size");
    if ((uint64_t)n > kMaxPoints) return fail(PGEOF_ERR_INVALID_ARGUMENT, std::string(what) + " exceeds 2^32-2 points");
    return PGEOF_OK;
}

int check_csr(int64_t n_xyz, int64_t nnz, int64_t n_points) {
    PGEOF_TRY(check_cloud(n_xyz, "xyz"));
    if (n_points < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn_ptr must hold at least one entry");
    if ((uint64_t)n_points > kMaxPoints) return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn_ptr is too long");
    if (nnz < 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn has a negative size");
    return PGEOF_OK;
}

// include/pgeof.hpp:123-132
bool check_scales(const uint32_t* k_scales, int64_t n) {
    uint32_t prev = 1;
    for (int64_t i = 0; i < n; ++i) {
        if (k_scales[i] < prev) return false;
        prev = k_scales[i];
    }
    return true;
}

// ------------------------------------------------------------ device impls
int knn_impl(const float* data, uint64_t n_data, const float* query, uint64_t n_query, uint32_t knn,
             uint32_t* indices, float* sqr_dist, bool query_is_data, cudaStream_t s) {
    if (n_query == 0 || knn == 0) return PGEOF_OK;
    GridIndex<float> grid;
    PGEOF_TRY(build_grid<float>(data, n_data, knn, 0.0f, 0.0f, grid, s));
    SPoint<float>* q = grid.pts;
    const uint32_t* qstart = grid.cell_start;
    Scratch qmem, qstart_mem;
    if (!query_is_data) {
        PGEOF_TRY(sort_queries<float>(query, n_query, grid.g, qmem, &q, qstart_mem, s));
        qstart = qstart_mem.as<uint32_t>();
    }
    SearchOut<float> out;
    out.indices = indices;
    out.sqr_dist = sqr_dist;
    return launch_search<float>(grid, q, qstart, n_query, MODE_KNN, knn, 0.0f, out, s);
}

int radius_impl(const float* data, uint64_t n_data, const float* query, uint64_t n_query, float radius,
                uint32_t max_knn, int32_t* indices, float* sqr_dist, bool query_is_data, cudaStream_t s,
                uint32_t* found = nullptr) {
    if (n_query == 0 || max_knn == 0) return PGEOF_OK;
    GridIndex<float> grid;
    const float r = std::fabs(radius);
    PGEOF_TRY(build_grid<float>(data, n_data, max_knn, r / 4.0f, r, grid, s));
    SPoint<float>* q = grid.pts;
    const uint32_t* qstart = grid.cell_start;
    Scratch qmem, qstart_mem;
    if (!query_is_data) {
        PGEOF_TRY(sort_queries<float>(query, n_query, grid.g, qmem, &q, qstart_mem, s));
        qstart = qstart_mem.as<uint32_t>();
    }
    SearchOut<float> out;
    out.indices = indices;
    out.sqr_dist = sqr_dist;
    out.radius_fill_last = true;
    out.found = found;
    return launch_search<float>(grid, q, qstart, n_query, MODE_RADIUS, max_knn, radius, out, s);
}

int features_impl(const float* xyz, uint64_t n_xyz, const uint32_t* nn, uint64_t nnz, const uint32_t* nn_ptr,
                  uint64_t n_points, int kind, uint64_t k_min, const uint32_t* scales, int64_t n_scales,
                  uint32_t k_step, uint32_t k_min_search, float* out, cudaStream_t s) {
    if (n_points == 0) return PGEOF_OK;
    Scratch xyz4;
    PGEOF_TRY(xyz4.alloc(std::max<uint64_t>(n_xyz, 1) * sizeof(float4), s));
    PGEOF_TRY(pad_xyz(xyz, n_xyz, xyz4.as<float4>(), s));
    if (kind == 2)
        return launch_optimal(xyz4.as<float4>(), n_xyz, nn, nnz, nn_ptr, n_points, (uint32_t)k_min, k_step,
                              k_min_search, out, nullptr, s);
    if (kind == 1 && n_scales == 0) return PGEOF_OK;
    // Clouds larger than L2 (16 B per point against 129 MB, from 8M points):
    // rows in the spatial order of their first neighbour, so that the rows a
    // block processes gather from the same region of the cloud -- 16M points,
    // k = 50: 24.4 -> 15.2 ms; at 1M-4M points the ordering costs more than it
    // saves. PGEOF_ROW_ORDER_POINTS overrides the threshold (0: never).
    static const uint64_t reorder_from = [] {
        const char* e = getenv("PGEOF_ROW_ORDER_POINTS");
        return e ? (uint64_t)strtoull(e, nullptr, 10) : (uint64_t)8000000;
    }();
    if (reorder_from > 0 && n_xyz >= reorder_from && n_points >= 65536) {
        Scratch rxyz;
        PGEOF_TRY(rxyz.alloc(n_points * 3 * sizeof(float), s));
        PGEOF_TRY(first_neighbour_xyz(xyz, n_xyz, nn, nnz, nn_ptr, n_points, rxyz.as<float>(), s));
        GridIndex<float> rows;
        if (build_grid<float>(rxyz.as<float>(), n_points, 8, 0.0f, 0.0f, rows, s) == PGEOF_OK)
            return launch_features(xyz4.as<float4>(), n_xyz, nn, nnz, nn_ptr, n_points, kind == 0, k_min, scales,
                                   (int)n_scales, out, nullptr, s, nullptr, 0, rows.pts, 0, 0, true);
        // (a cloud the grid cannot order, e.g. non-finite coordinates: plain order)
    }
    return launch_features(xyz4.as<float4>(), n_xyz, nn, nnz, nn_ptr, n_points, kind == 0, k_min, scales,
                           (int)n_scales, out, nullptr, s);
}

// include/pgeof.hpp:325-375 on an existing grid of xyz: the radius search
// hands each query's nearest min(found, max_knn) straight to PCA and the
// selected features (no neighbour table). Feature lists longer than one
// launch's share run the search once per share of ids.
template <typename T>
int selected_on_grid(const GridIndex<T>& grid, const T* xyz, uint64_t n, T radius, uint32_t max_knn,
                     const int32_t* ids, int64_t n_ids, T* out, cudaStream_t s) {
    if (n >= 0xffffffffull) return fail(PGEOF_ERR_INVALID_ARGUMENT, "compute_features_selected: too many points");
    const uint32_t k_search = std::max<uint32_t>(max_knn, 1u);
    SelSpec<T> sp;
    Scratch xyz4;
    if constexpr (sizeof(T) == sizeof(float)) {
        // one 16-byte gather per neighbour instead of three 4-byte ones
        PGEOF_TRY(xyz4.alloc(n * sizeof(float4), s));
        PGEOF_TRY(pad_xyz(reinterpret_cast<const float*>(xyz), n, xyz4.as<float4>(), s));
        sp.xyz4 = xyz4.as<float4>();
    } else {
        sp.xyz = xyz;
    }
    sp.out = out;
    sp.max_knn = max_knn;
    sp.out_stride = (uint32_t)n_ids;
    sp.order = eig_order();
    sp.ring = sel_ring_slots(k_search);
    SearchOut<T> so;
    so.radius_fill_last = false;
    so.sel = &sp;
    for (int64_t off = 0; off < n_ids; off += kSelMaxIds) {
        sp.id_offset = (uint32_t)off;
        sp.n_ids = (int)std::min<int64_t>(kSelMaxIds, n_ids - off);
        for (int t = 0; t < sp.n_ids; ++t) sp.ids[t] = ids[off + t];
        PGEOF_TRY(launch_search<T>(grid, grid.pts, grid.cell_start, n, MODE_RADIUS, k_search, radius, so, s));
    }
    return PGEOF_OK;
}

template <typename T>
int selected_impl(const T* xyz, uint64_t n, T radius, uint32_t max_knn, const int32_t* ids, int64_t n_ids, T* out,
                  cudaStream_t s) {
    if (n == 0 || n_ids == 0) return PGEOF_OK;
    GridIndex<T> grid;
    const float r = (float)std::fabs((double)radius);
    PGEOF_TRY(build_grid<T>(xyz, n, std::max<uint32_t>(max_knn, 1u), r / 4.0f, r, grid, s));
    return selected_on_grid<T>(grid, xyz, n, radius, max_knn, ids, n_ids, out, s);
}

}  // namespace

// ------------------------------------------------------------ kernel timing
std::atomic<int> g_profile_on{0};
namespace {
struct TimedLaunch {
    const char* name;
    cudaEvent_t a, b;
};
std::mutex g_prof_mu;
std::vector<TimedLaunch> g_prof;
std::vector<cudaEvent_t> g_event_pool;

cudaEvent_t take_event() {
    {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        if (!g_event_pool.empty()) {
            cudaEvent_t e = g_event_pool.back();
            g_event_pool.pop_back();
            return e;
        }
    }
    cudaEvent_t e = nullptr;
    if (cudaEventCreate(&e) != cudaSuccess) {
        (void)cudaGetLastError();
        return nullptr;
    }
    return e;
}
}  // namespace

KernelTimer::KernelTimer(const char* kernel_name, cudaStream_t stream) : name(kernel_name), s(stream) {
    if (g_profile_on.load(std::memory_order_relaxed)) {
        a = take_event();
        if (a) cudaEventRecord(a, s);
    }
}

KernelTimer::~KernelTimer() {
    if (!a) return;
    cudaEvent_t b = take_event();
    if (!b) return;
    cudaEventRecord(b, s);
    std::lock_guard<std::mutex> lk(g_prof_mu);
    g_prof.push_back({name, a, b});
}

void set_error(const std::string& msg) { t_last_error = msg; }
int fail(int status, const std::string& msg) {
    t_last_error = msg;
    return status;
}
int check_launch(const char* what) {
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return fail(PGEOF_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return PGEOF_OK;
}
int current_device_info(const DeviceInfo** out) {
    DevState* st;
    PGEOF_TRY(device_state(&st));
    *out = &st->info;
    return PGEOF_OK;
}
uint32_t* device_error_word() {
    if (t_error_word_override) return t_error_word_override;
    DevState* st = nullptr;
    if (device_state(&st) != PGEOF_OK) return nullptr;
    return st->err_word;
}
int scratch_alloc(void** p, size_t bytes, cudaStream_t s) {
    DevState* st;
    PGEOF_TRY(device_state(&st));
    PGEOF_CUDA_TRY(cudaMallocFromPoolAsync(p, bytes, st->pool, s));
    count_device_alloc();
    return PGEOF_OK;
}
void scratch_free(void* p, cudaStream_t s) { cudaFreeAsync(p, s); }
int eig_order() { return g_eig_order.load(std::memory_order_relaxed); }

}  // namespace pgeof

using namespace pgeof;

namespace {
bool page_locked(const void* p) {
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return at.type == cudaMemoryTypeHost;
}

// A block of the page-locked host cache, returned to it on scope exit.
struct HostBlock {
    void* p = nullptr;
    ~HostBlock() {
        if (p) pgeof_host_free(p);
    }
    int alloc(size_t bytes) { return pgeof_host_alloc(bytes, &p); }
};

template <typename T>
int host_selected(const T* xyz, int64_t n, T radius, uint32_t max_knn, const int32_t* ids, int64_t n_ids,
                         T* features) {
    PGEOF_TRY(check_cloud(n, "xyz"));
    if (n_ids < 0 || (n_ids > 0 && !ids)) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid selected feature list");
    if (n == 0 || n_ids == 0) return PGEOF_OK;
    // Pageable caller arrays are staged through page-locked blocks: the copies
    // then run asynchronously at full speed, and concurrent calls (a request
    // server's slots) do not queue on the driver's own pageable staging.
    const uint64_t cnt = (uint64_t)n * n_ids;
    HostBlock in_stage, out_stage;
    const T* src = xyz;
    T* dst = features;
    if (!page_locked(xyz) && in_stage.alloc(3ull * n * sizeof(T)) == PGEOF_OK) {
        std::memcpy(in_stage.p, xyz, 3ull * n * sizeof(T));
        src = static_cast<const T*>(in_stage.p);
    }
    if (!page_locked(features) && out_stage.alloc(cnt * sizeof(T)) == PGEOF_OK) dst = static_cast<T*>(out_stage.p);
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    Scratch d_xyz, d_out;
    const int st = [&] {
        PGEOF_TRY(upload(d_xyz, src, 3ull * n, s));
        PGEOF_TRY(d_out.alloc(cnt * sizeof(T), s));
        PGEOF_TRY(selected_impl<T>(d_xyz.as<T>(), n, radius, max_knn, ids, n_ids, d_out.as<T>(), s));
        PGEOF_TRY(download(dst, d_out, cnt, s));
        return finish_host(ce, s);
    }();
    if (st != PGEOF_OK) {
        cudaStreamSynchronize(s);  // no copy may still touch the staging blocks
        return st;
    }
    if (dst != features) std::memcpy(features, dst, cnt * sizeof(T));
    return PGEOF_OK;
}

struct OccEntry {
    int device;
    const void* kernel;
    int threads, smem, per_sm;
};
std::mutex g_occ_mu;
std::vector<OccEntry> g_occ;
// Largest dynamic shared memory limit set on each (device, kernel): the limit
// is only ever raised, so a launch whose size was cached earlier stays valid
// after launches of the same kernel with other sizes.
struct SmemLimit {
    int device;
    const void* kernel;
    int limit;
};
std::vector<SmemLimit> g_smem_limit;
// Shared-memory carveout preference last set on each (device, kernel) (-1:
// the driver's default).
struct CarveEntry {
    int device;
    const void* kernel;
    int carveout;
};
std::vector<CarveEntry> g_carve;

// Cache of page-locked host blocks behind pgeof_host_alloc / pgeof_host_free.
struct HostPool {
    std::mutex mu;
    std::multimap<size_t, void*> free_blocks;  // size -> block
    std::unordered_map<void*, size_t> size_of;  // every block handed out or cached
    size_t cached = 0;
    size_t cap = 0;
    bool cap_read = false;
};
HostPool& host_pool() {
    static HostPool* p = new HostPool();  // never destroyed: blocks may outlive static teardown
    return *p;
}
size_t host_pool_cap(HostPool& hp) {
    if (!hp.cap_read) {
        hp.cap = (size_t)8 << 30;
        if (const char* e = getenv("PGEOF_HOST_POOL_BYTES")) hp.cap = (size_t)strtoull(e, nullptr, 10);
        hp.cap_read = true;
    }
    return hp.cap;
}

}  // namespace

int pgeof::kernel_blocks_per_sm(const void* kernel, int threads, int smem, int* per_sm) {
    int dev = 0;
    PGEOF_CUDA_TRY(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(g_occ_mu);
    for (const OccEntry& e : g_occ)
        if (e.device == dev && e.kernel == kernel && e.threads == threads && e.smem == smem) {
            *per_sm = e.per_sm;
            return PGEOF_OK;
        }
    if (smem > 48 * 1024) {
        SmemLimit* lim = nullptr;
        for (SmemLimit& l : g_smem_limit)
            if (l.device == dev && l.kernel == kernel) lim = &l;
        if (!lim) {
            g_smem_limit.push_back(SmemLimit{dev, kernel, 48 * 1024});
            lim = &g_smem_limit.back();
        }
        if (smem > lim->limit) {
            PGEOF_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
            lim->limit = smem;
        }
    }
    int n = 0;
    PGEOF_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, smem));
    n = std::max(n, 1);
    g_occ.push_back(OccEntry{dev, kernel, threads, smem, n});
    *per_sm = n;
    return PGEOF_OK;
}

int pgeof::cap_smem_carveout(const void* kernel, int threads, int smem) {
    int per_sm = 0;
    PGEOF_TRY(kernel_blocks_per_sm(kernel, threads, smem, &per_sm));
    int dev = 0;
    PGEOF_CUDA_TRY(cudaGetDevice(&dev));
    // 1 KB of shared memory is reserved per resident block
    const int want = (size_t)per_sm * ((size_t)smem + 1024) > (size_t)196 * 1024 ? 85 : -1;
    std::lock_guard<std::mutex> lk(g_occ_mu);
    CarveEntry* cur = nullptr;
    for (CarveEntry& e : g_carve)
        if (e.device == dev && e.kernel == kernel) cur = &e;
    if (!cur) {
        g_carve.push_back(CarveEntry{dev, kernel, -1});
        cur = &g_carve.back();
    }
    if (cur->carveout != want) {
        PGEOF_CUDA_TRY(cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, want));
        cur->carveout = want;
    }
    return PGEOF_OK;
}

// =========================================================================
// ------------------------------------------------ resident clouds (serve.cu)
int pgeof::resident_cloud_build(const float* xyz, uint64_t n, float radius_hint, uint32_t k_hint,
                                ResidentCloud& out) {
    if (n == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "a resident cloud needs at least one point");
    PGEOF_TRY(check_cloud((int64_t)n, "xyz"));
    const cudaStream_t s = host_stream();
    out.n = n;
    PGEOF_TRY(upload(out.xyz, xyz, 3ull * n, s));
    const float r = std::fabs(radius_hint);
    PGEOF_TRY(build_grid<float>(out.xyz.as<float>(), n, std::max<uint32_t>(k_hint, 1u), r / 4.0f, r, out.grid, s));
    PGEOF_CUDA_TRY(cudaStreamSynchronize(s));  // complete before any other stream reads it
    return PGEOF_OK;
}

int pgeof::host_selected_resident(const ResidentCloud& c, float radius, uint32_t max_knn, const int32_t* ids,
                                  int64_t n_ids, float* features) {
    if (n_ids < 0 || (n_ids > 0 && !ids)) return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid selected feature list");
    if (c.n == 0 || n_ids == 0) return PGEOF_OK;
    const uint64_t cnt = c.n * (uint64_t)n_ids;
    HostBlock out_stage;
    float* dst = features;
    if (!page_locked(features) && out_stage.alloc(cnt * sizeof(float)) == PGEOF_OK)
        dst = static_cast<float*>(out_stage.p);
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    Scratch d_out;
    const int st = [&] {
        PGEOF_TRY(d_out.alloc(cnt * sizeof(float), s));
        PGEOF_TRY(selected_on_grid<float>(c.grid, c.xyz.as<float>(), c.n, radius, max_knn, ids, n_ids,
                                          d_out.as<float>(), s));
        PGEOF_TRY(download(dst, d_out, cnt, s));
        return finish_host(ce, s);
    }();
    if (st != PGEOF_OK) {
        cudaStreamSynchronize(s);
        return st;
    }
    if (dst != features) std::memcpy(features, dst, cnt * sizeof(float));
    return PGEOF_OK;
}

extern "C" {

int pgeof_abi_version(void) { return PGEOF_ABI_VERSION; }

const char* pgeof_status_string(int status) {
    switch (status) {
        case PGEOF_OK: return "ok";
        case PGEOF_ERR_INVALID_ARGUMENT: return "invalid argument";
        case PGEOF_ERR_DATA: return "invalid neighbour data";
        case PGEOF_ERR_OUT_OF_MEMORY: return "out of device memory";
        case PGEOF_ERR_CUDA: return "CUDA error";
        case PGEOF_ERR_NO_DEVICE: return "no usable GB300 device";
        case PGEOF_ERR_INTERNAL: return "internal bound exceeded";
        default: return "unknown status";
    }
}

const char* pgeof_last_error_message(void) { return t_last_error.c_str(); }

uint64_t pgeof_kernel_launch_count(void) { return g_launch_count.load(); }
uint64_t pgeof_device_alloc_count(void) { return g_device_alloc_count.load(); }

int pgeof_set_eig_order(int order) {
    if (order != 0 && order != 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "eig order must be 0 or 1");
    g_eig_order.store(order);
    return PGEOF_OK;
}
int pgeof_get_eig_order(void) { return g_eig_order.load(); }

int pgeof_profile_enable(int on) {
    g_profile_on.store(on ? 1 : 0);
    return PGEOF_OK;
}

int pgeof_profile_report(char* buf, size_t buf_len) {
    std::vector<TimedLaunch> rec;
    {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        rec.swap(g_prof);
    }
    struct Agg {
        std::string name;
        uint64_t n = 0;
        double ms = 0.0;
    };
    std::vector<Agg> agg;
    int status = PGEOF_OK;
    for (const TimedLaunch& t : rec) {
        float ms = 0.0f;
        cudaError_t e = cudaEventSynchronize(t.b);
        if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, t.a, t.b);
        if (e != cudaSuccess) {
            (void)cudaGetLastError();
            status = fail(PGEOF_ERR_CUDA, std::string("kernel timing: ") + cudaGetErrorString(e));
            continue;
        }
        auto it = std::find_if(agg.begin(), agg.end(), [&](const Agg& x) { return x.name == t.name; });
        if (it == agg.end()) {
            agg.push_back({t.name, 0, 0.0});
            it = agg.end() - 1;
        }
        it->n += 1;
        it->ms += ms;
    }
    {
        std::lock_guard<std::mutex> lk(g_prof_mu);
        for (const TimedLaunch& t : rec) {
            g_event_pool.push_back(t.a);
            g_event_pool.push_back(t.b);
        }
    }
    std::string out;
    for (const Agg& x : agg) {
        char line[256];
        snprintf(line, sizeof(line), "%s %llu %.6f\n", x.name.c_str(), (unsigned long long)x.n, x.ms);
        out += line;
    }
    if (buf && buf_len) {
        const size_t n = std::min(out.size(), buf_len - 1);
        memcpy(buf, out.data(), n);
        buf[n] = '\0';
    }
    return status;
}

int pgeof_take_device_errors(pgeof_stream_t stream, uint32_t* bits) {
    DevState* st;
    PGEOF_TRY(device_state(&st));
    PGEOF_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    uint32_t v = 0, v_noalloc = 0;
    PGEOF_CUDA_TRY(cudaMemcpy(&v, st->err_word, sizeof(v), cudaMemcpyDeviceToHost));
    PGEOF_CUDA_TRY(cudaMemset(st->err_word, 0, sizeof(v)));
    PGEOF_TRY(noalloc_take_errors(&v_noalloc));
    if (bits) *bits = v | v_noalloc;
    return PGEOF_OK;
}

// ---------------------------------------------------------------- host block cache

int pgeof_host_alloc(size_t bytes, void** ptr) {
    if (!ptr) return fail(PGEOF_ERR_INVALID_ARGUMENT, "pgeof_host_alloc: ptr is NULL");
    *ptr = nullptr;
    constexpr size_t kGranule = (size_t)2 << 20;
    const size_t want = (std::max<size_t>(bytes, 1) + kGranule - 1) / kGranule * kGranule;
    HostPool& hp = host_pool();
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        auto it = hp.free_blocks.lower_bound(want);
        if (it != hp.free_blocks.end() && it->first <= want + want / 4) {
            *ptr = it->second;
            hp.cached -= it->first;
            hp.free_blocks.erase(it);
            return PGEOF_OK;
        }
    }
    DevState* st;
    PGEOF_TRY(device_state(&st));
    void* p = nullptr;
    PGEOF_CUDA_TRY(cudaHostAlloc(&p, want, cudaHostAllocPortable));
    std::lock_guard<std::mutex> lk(hp.mu);
    hp.size_of[p] = want;
    *ptr = p;
    return PGEOF_OK;
}

int pgeof_host_free(void* ptr) {
    if (!ptr) return PGEOF_OK;
    HostPool& hp = host_pool();
    bool release = false;
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        auto it = hp.size_of.find(ptr);
        if (it == hp.size_of.end()) return fail(PGEOF_ERR_INVALID_ARGUMENT, "pgeof_host_free: not a pgeof host block");
        const size_t sz = it->second;
        if (hp.cached + sz <= host_pool_cap(hp)) {
            hp.free_blocks.emplace(sz, ptr);
            hp.cached += sz;
        } else {
            hp.size_of.erase(it);
            release = true;
        }
    }
    if (release) PGEOF_CUDA_TRY(cudaFreeHost(ptr));
    return PGEOF_OK;
}

int pgeof_host_pool_trim(void) {
    HostPool& hp = host_pool();
    std::vector<void*> out;
    {
        std::lock_guard<std::mutex> lk(hp.mu);
        for (auto& kv : hp.free_blocks) {
            out.push_back(kv.second);
            hp.size_of.erase(kv.second);
        }
        hp.free_blocks.clear();
        hp.cached = 0;
    }
    for (void* p : out) PGEOF_CUDA_TRY(cudaFreeHost(p));
    return PGEOF_OK;
}

// ---------------------------------------------------------------- device API
int pgeof_knn_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query, uint32_t knn,
                         uint32_t* indices, float* sqr_dist, pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n_data, "data"));
    PGEOF_TRY(check_cloud(n_query, "query"));
    if ((int64_t)knn > n_data)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size");
    return knn_impl(data, n_data, query, n_query, knn, indices, sqr_dist, data == query && n_data == n_query,
                    (cudaStream_t)stream);
}

int pgeof_radius_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                            float search_radius, uint32_t max_knn, int32_t* indices, float* sqr_dist,
                            pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n_data, "data"));
    PGEOF_TRY(check_cloud(n_query, "query"));
    if ((int64_t)max_knn > n_data)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "max knn size is greater than the data point cloud size");
    return radius_impl(data, n_data, query, n_query, search_radius, max_knn, indices, sqr_dist,
                       data == query && n_data == n_query, (cudaStream_t)stream);
}

int pgeof_radius_search_csr_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                                float search_radius, uint32_t max_knn, uint32_t* nn, uint32_t* nn_ptr,
                                pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n_data, "data"));
    PGEOF_TRY(check_cloud(n_query, "query"));
    if ((int64_t)max_knn > n_data)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "max knn size is greater than the data point cloud size");
    if ((uint64_t)n_query * max_knn >= 0xffffffffull)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "n_query * max_knn must stay below 2^32 for uint32 nn_ptr");
    if (!nn_ptr || (!nn && n_query > 0 && max_knn > 0))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "nn and nn_ptr must not be NULL");
    cudaStream_t s = (cudaStream_t)stream;
    const uint64_t m = (uint64_t)n_query;
    if (m == 0 || max_knn == 0) {
        PGEOF_CUDA_TRY(cudaMemsetAsync(nn_ptr, 0, (m + 1) * sizeof(uint32_t), s));
        return PGEOF_OK;
    }
    Scratch table, found, counts, partials;
    PGEOF_TRY(table.alloc(m * max_knn * sizeof(int32_t), s));
    PGEOF_TRY(found.alloc(m * sizeof(uint32_t), s));
    PGEOF_TRY(counts.alloc(m * sizeof(uint32_t), s));
    PGEOF_TRY(partials.alloc((m / 1024 + 1) * sizeof(uint32_t), s));
    PGEOF_TRY(radius_impl(data, n_data, query, n_query, search_radius, max_knn, table.as<int32_t>(), nullptr,
                          data == query && n_data == n_query, s, found.as<uint32_t>()));
    return launch_csr_from_table(table.as<int32_t>(), found.as<uint32_t>(), m, max_knn, counts.as<uint32_t>(),
                                 partials.as<uint32_t>(), nn_ptr, nn, s);
}

int pgeof_compute_features_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                               const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, float* features,
                               pgeof_stream_t stream) {
    if (k_min < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min should be > 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return features_impl(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 0, k_min, nullptr, 0, 0, 0, features,
                         (cudaStream_t)stream);
}

int pgeof_compute_features_multiscale_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                          const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                          int64_t n_scales, float* features, pgeof_stream_t stream) {
    if (n_scales < 0 || (n_scales > 0 && !k_scales) || !check_scales(k_scales, n_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return features_impl(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 1, 1, k_scales, n_scales, 0, 0, features,
                         (cudaStream_t)stream);
}

int pgeof_knn_features_f32(const float* xyz, int64_t n, uint32_t knn, const uint32_t* k_scales, int64_t n_scales,
                           float* features, pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n, "xyz"));
    if (knn == 0) return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn should be >= 1");
    if ((int64_t)knn > n) return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size");
    if (n_scales < 0 || (n_scales > 0 && !k_scales) || !check_scales(k_scales, n_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    if (n_scales > 0 && k_scales[n_scales - 1] > knn)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales must not exceed knn");
    if (n == 0) return PGEOF_OK;
    cudaStream_t s = (cudaStream_t)stream;
    GridIndex<float> grid;
    PGEOF_TRY(build_grid<float>(xyz, (uint64_t)n, knn, 0.0f, 0.0f, grid, s));
    // neighbour rows in cell order (no distances): the feature pass then walks
    // spatially adjacent rows, whose neighbourhoods overlap in L1
    Scratch nn, xyz4;
    PGEOF_TRY(nn.alloc((size_t)n * knn * sizeof(uint32_t), s));
    SearchOut<float> o;
    o.indices = nn.p;
    o.sqr_dist = nullptr;
    o.rows_in_query_order = true;
    PGEOF_TRY(launch_search<float>(grid, grid.pts, grid.cell_start, (uint64_t)n, MODE_KNN, knn, 0.0f, o, s));
    PGEOF_TRY(xyz4.alloc((size_t)n * sizeof(float4), s));
    PGEOF_TRY(pad_xyz(xyz, (uint64_t)n, xyz4.as<float4>(), s));
    return launch_features(xyz4.as<float4>(), (uint64_t)n, nn.as<uint32_t>(), (uint64_t)n * knn, nullptr,
                           (uint64_t)n, n_scales == 0, 1, k_scales, (int)n_scales, features, nullptr, s, nullptr, 0,
                           grid.pts, knn);
}

int pgeof_compute_features_optimal_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                       const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min, uint32_t k_step,
                                       uint32_t k_min_search, float* features, pgeof_stream_t stream) {
    if (k_min < 1 && k_min_search < 1)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min and k_min_search should be > 1");
    if (k_step < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_step should be >= 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return features_impl(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 2, k_min, nullptr, 0, k_step, k_min_search,
                         features, (cudaStream_t)stream);
}

int pgeof_compute_features_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                               const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, double* features,
                               pgeof_stream_t stream) {
    if (k_min < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min should be > 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return launch_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 0, k_min, nullptr, 0, 0, 0, features,
                               (cudaStream_t)stream);
}

int pgeof_compute_features_multiscale_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                          const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                          int64_t n_scales, double* features, pgeof_stream_t stream) {
    if (n_scales < 0 || n_scales > (1 << 20) || (n_scales > 0 && !k_scales) || !check_scales(k_scales, n_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return launch_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 1, 1, k_scales, (int)n_scales, 0, 0,
                               features, (cudaStream_t)stream);
}

int pgeof_compute_features_optimal_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                       const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min, uint32_t k_step,
                                       uint32_t k_min_search, double* features, pgeof_stream_t stream) {
    if (k_min < 1 && k_min_search < 1)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min and k_min_search should be > 1");
    if (k_step < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_step should be >= 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return launch_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 2, k_min, nullptr, 0, k_step, k_min_search,
                               features, (cudaStream_t)stream);
}

int pgeof_compute_features_selected_f32(const float* xyz, int64_t n, float search_radius, uint32_t max_knn,
                                        const int32_t* selected, int64_t n_selected, float* features,
                                        pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n, "xyz"));
    if (n_selected < 0 || (n_selected > 0 && !selected))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid selected feature list");
    return selected_impl<float>(xyz, n, search_radius, max_knn, selected, n_selected, features,
                                (cudaStream_t)stream);
}

int pgeof_compute_features_selected_f64(const double* xyz, int64_t n, double search_radius, uint32_t max_knn,
                                        const int32_t* selected, int64_t n_selected, double* features,
                                        pgeof_stream_t stream) {
    PGEOF_TRY(check_cloud(n, "xyz"));
    if (n_selected < 0 || (n_selected > 0 && !selected))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "invalid selected feature list");
    return selected_impl<double>(xyz, n, search_radius, max_knn, selected, n_selected, features,
                                 (cudaStream_t)stream);
}

// ---------------------------------------------------------------- host API
// First row of chunk c of a C-chunk host pipeline over m rows (equal chunks:
// a half-size first chunk, so that the first transfer starts earlier,
// measured slower on the 1M-point scene -- kNN 3.07 -> 3.21 ms, multiscale
// 1.61 -> 1.74 ms).
static uint64_t pipeline_row(uint64_t m, int c, int C) { return m * (uint64_t)c / (uint64_t)C; }

int pgeof_host_knn_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                              uint32_t knn, uint32_t* indices, float* sqr_dist) {
    PGEOF_TRY(check_cloud(n_data, "data"));
    PGEOF_TRY(check_cloud(n_query, "query"));
    if ((int64_t)knn > n_data)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "knn size is greater than the data point cloud size");
    if (n_query == 0 || knn == 0) return PGEOF_OK;
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    const bool same = data == query && n_data == n_query;
    Scratch d_data, d_query, d_idx, d_d2;
    PGEOF_TRY(upload(d_data, data, 3ull * n_data, s));
    if (!same) PGEOF_TRY(upload(d_query, query, 3ull * n_query, s));
    const uint64_t cnt = (uint64_t)n_query * knn;
    PGEOF_TRY(d_idx.alloc(cnt * sizeof(uint32_t), s));
    PGEOF_TRY(d_d2.alloc(cnt * sizeof(float), s));
    const uint64_t out_bytes = cnt * (sizeof(uint32_t) + sizeof(float));
    if (out_bytes < (128ull << 20) || n_query < 65536) {
        PGEOF_TRY(knn_impl(d_data.as<float>(), n_data, same ? d_data.as<float>() : d_query.as<float>(), n_query, knn,
                           d_idx.as<uint32_t>(), d_d2.as<float>(), same, s));
        PGEOF_TRY(download(indices, d_idx, cnt, s));
        PGEOF_TRY(download(sqr_dist, d_d2, cnt, s));
        return finish_host(ce, s);
    }
    // Large results: the queries in chunks of consecutive rows, each sorted into
    // cell order and searched against the one grid, so that chunk c's rows
    // download while chunk c+1 is searched.
    GridIndex<float> grid;
    PGEOF_TRY(build_grid<float>(d_data.as<float>(), (uint64_t)n_data, knn, 0.0f, 0.0f, grid, s));
    const float* qbase = same ? d_data.as<float>() : d_query.as<float>();
    const cudaStream_t cout = host_copy_stream(1);
    const int C = (int)std::min<uint64_t>(8, std::max<uint64_t>(2, out_bytes / (96ull << 20)));
    std::vector<cudaEvent_t> ev(C + 2, nullptr);  // start, one per chunk, final
    for (auto& e : ev) PGEOF_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    int status = PGEOF_OK;
    Scratch qmem, qstart_mem;
    const uint64_t m = (uint64_t)n_query;
    if (cudaEventRecord(ev[0], s) != cudaSuccess || cudaStreamWaitEvent(cout, ev[0], 0) != cudaSuccess)
        status = fail(PGEOF_ERR_CUDA, "knn pipeline: stream ordering failed");
    for (int c = 0; c < C && status == PGEOF_OK; ++c) {
        const uint64_t r0 = pipeline_row(m, c, C), r1 = pipeline_row(m, c + 1, C);
        if (r1 == r0) continue;
        SPoint<float>* qs = nullptr;
        status = sort_queries<float>(qbase + 3 * r0, r1 - r0, grid.g, qmem, &qs, qstart_mem, s);
        if (status != PGEOF_OK) break;
        SearchOut<float> o;
        o.indices = d_idx.as<uint32_t>() + r0 * knn;
        o.sqr_dist = d_d2.as<float>() + r0 * knn;
        status = launch_search<float>(grid, qs, qstart_mem.as<uint32_t>(), r1 - r0, MODE_KNN, knn, 0.0f, o, s);
        if (status != PGEOF_OK) break;
        if (cudaEventRecord(ev[1 + c], s) != cudaSuccess || cudaStreamWaitEvent(cout, ev[1 + c], 0) != cudaSuccess ||
            cudaMemcpyAsync(indices + r0 * knn, d_idx.as<uint32_t>() + r0 * knn, (r1 - r0) * knn * sizeof(uint32_t),
                            cudaMemcpyDeviceToHost, cout) != cudaSuccess ||
            cudaMemcpyAsync(sqr_dist + r0 * knn, d_d2.as<float>() + r0 * knn, (r1 - r0) * knn * sizeof(float),
                            cudaMemcpyDeviceToHost, cout) != cudaSuccess)
            status = fail(PGEOF_ERR_CUDA, "knn pipeline: download failed");
    }
    cudaEventRecord(ev[C + 1], cout);
    cudaStreamWaitEvent(s, ev[C + 1], 0);
    const int fin = finish_host(ce, s);
    for (auto& e : ev) cudaEventDestroy(e);
    return status != PGEOF_OK ? status : fin;
}

int pgeof_host_radius_search_f32(const float* data, int64_t n_data, const float* query, int64_t n_query,
                                 float search_radius, uint32_t max_knn, int32_t* indices, float* sqr_dist) {
    PGEOF_TRY(check_cloud(n_data, "data"));
    PGEOF_TRY(check_cloud(n_query, "query"));
    if ((int64_t)max_knn > n_data)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "max knn size is greater than the data point cloud size");
    if (n_query == 0 || max_knn == 0) return PGEOF_OK;
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    const bool same = data == query && n_data == n_query;
    Scratch d_data, d_query, d_idx, d_d2;
    PGEOF_TRY(upload(d_data, data, 3ull * n_data, s));
    if (!same) PGEOF_TRY(upload(d_query, query, 3ull * n_query, s));
    const uint64_t cnt = (uint64_t)n_query * max_knn;
    PGEOF_TRY(d_idx.alloc(cnt * sizeof(int32_t), s));
    PGEOF_TRY(d_d2.alloc(cnt * sizeof(float), s));
    PGEOF_TRY(radius_impl(d_data.as<float>(), n_data, same ? d_data.as<float>() : d_query.as<float>(), n_query,
                          search_radius, max_knn, d_idx.as<int32_t>(), d_d2.as<float>(), same, s));
    PGEOF_TRY(download(indices, d_idx, cnt, s));
    PGEOF_TRY(download(sqr_dist, d_d2, cnt, s));
    return finish_host(ce, s);
}

static int host_features(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz, const uint32_t* nn_ptr,
                         int64_t n_points, int kind, uint64_t k_min, const uint32_t* scales, int64_t n_scales,
                         uint32_t k_step, uint32_t k_min_search, float* features, uint64_t row_width) {
    if (n_points == 0 || row_width == 0) return PGEOF_OK;
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    Scratch d_xyz, d_nn, d_ptr, d_out;
    PGEOF_TRY(upload(d_xyz, xyz, 3ull * n_xyz, s));
    PGEOF_TRY(upload(d_ptr, nn_ptr, (uint64_t)n_points + 1, s));
    const uint64_t cnt = (uint64_t)n_points * row_width;
    PGEOF_TRY(d_out.alloc(cnt * sizeof(float), s));
    const uint64_t nn_bytes = (uint64_t)nnz * sizeof(uint32_t);
    if (kind == 2 || nn_bytes < (64ull << 20) || n_points < 1024) {
        PGEOF_TRY(upload(d_nn, nn, (uint64_t)nnz, s));
        PGEOF_TRY(features_impl(d_xyz.as<float>(), n_xyz, d_nn.as<uint32_t>(), nnz, d_ptr.as<uint32_t>(), n_points,
                                kind, k_min, scales, n_scales, k_step, k_min_search, d_out.as<float>(), s));
        PGEOF_TRY(download(features, d_out, cnt, s));
        return finish_host(ce, s);
    }
    // Large neighbour lists: rows in chunks, so that chunk c's neighbour upload,
    // chunk c-1's feature pass and chunk c-2's result download overlap. A chunk's
    // rows read only its own slice nn[nn_ptr[r0], nn_ptr[r1]) when nn_ptr is
    // non-decreasing (anything else is reported by the kernel as a data error);
    // the slices are clamped to len(nn) on the host.
    PGEOF_TRY(d_nn.alloc(nn_bytes, s));
    Scratch xyz4;
    PGEOF_TRY(xyz4.alloc(std::max<uint64_t>(n_xyz, 1) * sizeof(float4), s));
    PGEOF_TRY(pad_xyz(d_xyz.as<float>(), n_xyz, xyz4.as<float4>(), s));
    const cudaStream_t cin = host_copy_stream(0), cout = host_copy_stream(1);
    // ~24 MB of neighbour lists per chunk (1M-point k=50 multiscale through
    // the numpy API, repeated runs: 8 chunks 1.74-1.75 ms, 4 chunks 1.85-1.87
    // ms; single runs of 2 / 12 / 16 chunks 1.83 / 1.68 / 1.69 ms)
    const int C = (int)std::min<uint64_t>(8, std::max<uint64_t>(2, nn_bytes / (24ull << 20)));
    std::vector<cudaEvent_t> ev(2 * C + 3, nullptr);  // start, (upload, kernel) per chunk, 2 final
    for (auto& e : ev) PGEOF_CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    int status = PGEOF_OK;
    const uint64_t n = (uint64_t)n_points, total = (uint64_t)nnz;
    do {
        // scratch allocated on s must exist before the copy streams touch it
        if (cudaEventRecord(ev[0], s) != cudaSuccess || cudaStreamWaitEvent(cin, ev[0], 0) != cudaSuccess ||
            cudaStreamWaitEvent(cout, ev[0], 0) != cudaSuccess) {
            status = fail(PGEOF_ERR_CUDA, "feature pipeline: stream ordering failed");
            break;
        }
        for (int c = 0; c < C && status == PGEOF_OK; ++c) {
            const uint64_t r0 = pipeline_row(n, c, C), r1 = pipeline_row(n, c + 1, C);
            if (r1 == r0) continue;
            const uint64_t lo = std::min<uint64_t>(nn_ptr[r0], total);
            const uint64_t hi = std::min<uint64_t>(std::max<uint64_t>(nn_ptr[r1], lo), total);
            if (hi > lo &&
                cudaMemcpyAsync(d_nn.as<uint32_t>() + lo, nn + lo, (hi - lo) * sizeof(uint32_t),
                                cudaMemcpyHostToDevice, cin) != cudaSuccess) {
                status = fail(PGEOF_ERR_CUDA, "feature pipeline: upload failed");
                break;
            }
            if (cudaEventRecord(ev[1 + 2 * c], cin) != cudaSuccess ||
                cudaStreamWaitEvent(s, ev[1 + 2 * c], 0) != cudaSuccess) {
                status = fail(PGEOF_ERR_CUDA, "feature pipeline: stream ordering failed");
                break;
            }
            status = launch_features(xyz4.as<float4>(), n_xyz, d_nn.as<uint32_t>(), total, d_ptr.as<uint32_t>(),
                                     r1 - r0, kind == 0, k_min, scales, (int)n_scales, d_out.as<float>(), nullptr, s,
                                     nullptr, 0, nullptr, 0, r0);
            if (status != PGEOF_OK) break;
            if (cudaEventRecord(ev[2 + 2 * c], s) != cudaSuccess ||
                cudaStreamWaitEvent(cout, ev[2 + 2 * c], 0) != cudaSuccess ||
                cudaMemcpyAsync(features + r0 * row_width, d_out.as<float>() + r0 * row_width,
                                (r1 - r0) * row_width * sizeof(float), cudaMemcpyDeviceToHost, cout) != cudaSuccess) {
                status = fail(PGEOF_ERR_CUDA, "feature pipeline: download failed");
                break;
            }
        }
    } while (false);
    // the scratch is released on s: let s wait for both copy streams
    cudaEventRecord(ev[2 * C + 1], cin);
    cudaEventRecord(ev[2 * C + 2], cout);
    cudaStreamWaitEvent(s, ev[2 * C + 1], 0);
    cudaStreamWaitEvent(s, ev[2 * C + 2], 0);
    const int fin = finish_host(ce, s);
    for (auto& e : ev) cudaEventDestroy(e);
    return status != PGEOF_OK ? status : fin;
}

int pgeof_host_compute_features_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                    const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, float* features) {
    if (k_min < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min should be > 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 0, k_min, nullptr, 0, 0, 0, features, 11);
}

int pgeof_host_compute_features_multiscale_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                               const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                               int64_t n_scales, float* features) {
    if (n_scales < 0 || (n_scales > 0 && !k_scales) || !check_scales(k_scales, n_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 1, 1, k_scales, n_scales, 0, 0, features,
                         11ull * (uint64_t)n_scales);
}

int pgeof_host_compute_features_optimal_f32(const float* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                            const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min,
                                            uint32_t k_step, uint32_t k_min_search, float* features) {
    if (k_min < 1 && k_min_search < 1)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min and k_min_search should be > 1");
    if (k_step < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_step should be >= 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 2, k_min, nullptr, 0, k_step, k_min_search,
                         features, 12);
}

// Host-pointer float64 feature passes: upload, one kernel, download.
static int host_features_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                             const uint32_t* nn_ptr, int64_t n_points, int kind, uint64_t k_min,
                             const uint32_t* scales, int64_t n_scales, uint32_t k_step, uint32_t k_min_search,
                             double* features, uint64_t row_width) {
    if (n_points == 0 || row_width == 0) return PGEOF_OK;
    const cudaStream_t s = host_stream();
    CallErrors ce(s);
    PGEOF_TRY(ce.begin());
    Scratch d_xyz, d_nn, d_ptr, d_out;
    PGEOF_TRY(upload(d_xyz, xyz, 3ull * n_xyz, s));
    PGEOF_TRY(upload(d_nn, nn, (uint64_t)nnz, s));
    PGEOF_TRY(upload(d_ptr, nn_ptr, (uint64_t)n_points + 1, s));
    const uint64_t cnt = (uint64_t)n_points * row_width;
    PGEOF_TRY(d_out.alloc(cnt * sizeof(double), s));
    PGEOF_TRY(launch_features_f64(d_xyz.as<double>(), n_xyz, d_nn.as<uint32_t>(), nnz, d_ptr.as<uint32_t>(),
                                  n_points, kind, k_min, scales, (int)n_scales, k_step, k_min_search,
                                  d_out.as<double>(), s));
    PGEOF_TRY(download(features, d_out, cnt, s));
    return finish_host(ce, s);
}

int pgeof_host_compute_features_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                    const uint32_t* nn_ptr, int64_t n_points, uint64_t k_min, double* features) {
    if (k_min < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min should be > 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 0, k_min, nullptr, 0, 0, 0, features, 11);
}

int pgeof_host_compute_features_multiscale_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                               const uint32_t* nn_ptr, int64_t n_points, const uint32_t* k_scales,
                                               int64_t n_scales, double* features) {
    if (n_scales < 0 || n_scales > (1 << 20) || (n_scales > 0 && !k_scales) || !check_scales(k_scales, n_scales))
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_scales should be > 1 and sorted in ascending order");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 1, 1, k_scales, n_scales, 0, 0, features,
                             (uint64_t)n_scales * 11);
}

int pgeof_host_compute_features_optimal_f64(const double* xyz, int64_t n_xyz, const uint32_t* nn, int64_t nnz,
                                            const uint32_t* nn_ptr, int64_t n_points, uint32_t k_min,
                                            uint32_t k_step, uint32_t k_min_search, double* features) {
    if (k_min < 1 && k_min_search < 1)
        return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_min and k_min_search should be > 1");
    if (k_step < 1) return fail(PGEOF_ERR_INVALID_ARGUMENT, "k_step should be >= 1");
    PGEOF_TRY(check_csr(n_xyz, nnz, n_points));
    return host_features_f64(xyz, n_xyz, nn, nnz, nn_ptr, n_points, 2, k_min, nullptr, 0, k_step, k_min_search,
                             features, 12);
}

int pgeof_host_compute_features_selected_f32(const float* xyz, int64_t n, float search_radius, uint32_t max_knn,
                                             const int32_t* selected, int64_t n_selected, float* features) {
    return host_selected<float>(xyz, n, search_radius, max_knn, selected, n_selected, features);
}

int pgeof_host_compute_features_selected_f64(const double* xyz, int64_t n, double search_radius,
                                             uint32_t max_knn, const int32_t* selected, int64_t n_selected,
                                             double* features) {
    return host_selected<double>(xyz, n, search_radius, max_knn, selected, n_selected, features);
}

}  // extern "C"
