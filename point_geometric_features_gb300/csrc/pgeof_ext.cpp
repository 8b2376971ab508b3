// pgeof_ext.cpp -- the Python module `pgeof_ext`, a drop-in for pgeof's nanobind
// module (src/pgeof_ext.cpp:12-178): same function names, argument names,
// defaults, overload order, dtype strictness and error types, over the C ABI of
// libpgeof_cuda.so (include/pgeof_cuda.h).
//
// nanobind is not available here, so the module is built with pybind11 (the
// copy bundled with PyTorch). Behaviour kept from the reference:
//   * array arguments are "noconvert": a float64 xyz or int64 nn raises
//     TypeError instead of being cast (src/pgeof_ext.cpp:34-35);
//   * std::invalid_argument conditions raise ValueError with the reference's
//     messages;
//   * outputs are numpy arrays owned by Python. Their memory is a page-locked
//     block from the library's host cache (pgeof_host_alloc), returned to the
//     cache when the array is freed, so results arrive at DMA speed instead of
//     page-faulting fresh memory; PGEOF_HOST_POOL_BYTES=0 selects plain numpy
//     allocations.
// Differences: the GIL is released while the GPU works, and invalid CSR input
// (an nn index >= len(xyz), a decreasing nn_ptr) raises ValueError where the
// reference reads out of bounds.
//
// The `_dev_*` functions take raw device pointers (integers) and a CUDA stream;
// the package uses them for torch.cuda tensors.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "pgeof_cuda.h"

namespace py = pybind11;

namespace {

using f32arr = py::array_t<float, py::array::c_style>;
using f64arr = py::array_t<double, py::array::c_style>;
using u32arr = py::array_t<uint32_t, py::array::c_style>;

[[noreturn]] void raise_status(int st) {
    const std::string msg = pgeof_last_error_message();
    switch (st) {
        case PGEOF_ERR_INVALID_ARGUMENT:
        case PGEOF_ERR_DATA:
            throw py::value_error(msg);
        case PGEOF_ERR_OUT_OF_MEMORY:
            throw std::bad_alloc();
        default:
            throw std::runtime_error(std::string(pgeof_status_string(st)) + ": " + msg);
    }
}

inline void check(int st) {
    if (st != PGEOF_OK) raise_status(st);
}

bool use_host_cache() {
    static const bool on = [] {
        const char* e = getenv("PGEOF_HOST_POOL_BYTES");
        return !(e && strtoull(e, nullptr, 10) == 0);
    }();
    return on;
}

// A C-contiguous result array of `shape`, backed by a cached page-locked block.
template <typename T>
py::array_t<T, py::array::c_style> result_array(std::vector<int64_t> shape) {
    size_t count = 1;
    for (int64_t d : shape) count *= (size_t)std::max<int64_t>(d, 0);
    void* p = nullptr;
    if (count > 0 && use_host_cache() && pgeof_host_alloc(count * sizeof(T), &p) == PGEOF_OK) {
        py::capsule owner(p, [](void* q) { pgeof_host_free(q); });
        return py::array_t<T, py::array::c_style>(shape, static_cast<T*>(p), owner);
    }
    return py::array_t<T, py::array::c_style>(shape);
}

template <typename T>
int64_t cloud_rows(const py::array_t<T, py::array::c_style>& a, const char* name) {
    if (a.ndim() != 2 || a.shape(1) != 3)
        throw py::type_error(std::string(name) + " must be a C-contiguous (n, 3) array");
    return (int64_t)a.shape(0);
}

int64_t vec_len(const u32arr& a, const char* name) {
    if (a.ndim() != 1) throw py::type_error(std::string(name) + " must be a 1-D uint32 array");
    return (int64_t)a.shape(0);
}

void progress_done(bool verbose, int64_t n) {
    if (verbose) py::print(std::to_string(n) + " points done (GPU)");
}

// ------------------------------------------------------------------ numpy API
f32arr compute_features(const f32arr& xyz, const u32arr& nn, const u32arr& nn_ptr, size_t k_min, bool verbose) {
    const int64_t n_xyz = cloud_rows(xyz, "xyz");
    const int64_t nnz = vec_len(nn, "nn"), np1 = vec_len(nn_ptr, "nn_ptr");
    const int64_t n = np1 - 1;
    f32arr out = result_array<float>({std::max<int64_t>(n, 0), (int64_t)11});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_compute_features_f32(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n, (uint64_t)k_min,
                                             out.mutable_data());
    }
    check(st);
    progress_done(verbose, n);
    return out;
}

f32arr compute_features_multiscale(const f32arr& xyz, const u32arr& nn, const u32arr& nn_ptr,
                                   const std::vector<uint32_t>& k_scales, bool verbose) {
    const int64_t n_xyz = cloud_rows(xyz, "xyz");
    const int64_t nnz = vec_len(nn, "nn"), np1 = vec_len(nn_ptr, "nn_ptr");
    const int64_t n = np1 - 1;
    f32arr out = result_array<float>({std::max<int64_t>(n, 0), (int64_t)k_scales.size(), (int64_t)11});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_compute_features_multiscale_f32(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n,
                                                        k_scales.data(), (int64_t)k_scales.size(), out.mutable_data());
    }
    check(st);
    progress_done(verbose, n);
    return out;
}

f32arr compute_features_optimal(const f32arr& xyz, const u32arr& nn, const u32arr& nn_ptr, uint32_t k_min,
                                uint32_t k_step, uint32_t k_min_search, bool verbose) {
    const int64_t n_xyz = cloud_rows(xyz, "xyz");
    const int64_t nnz = vec_len(nn, "nn"), np1 = vec_len(nn_ptr, "nn_ptr");
    const int64_t n = np1 - 1;
    f32arr out = result_array<float>({std::max<int64_t>(n, 0), (int64_t)12});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_compute_features_optimal_f32(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n, k_min,
                                                     k_step, k_min_search, out.mutable_data());
    }
    check(st);
    progress_done(verbose, n);
    return out;
}

// float64 instantiations of the three CSR passes (kind 0 / 1 / 2)
f64arr features_f64(int kind, const f64arr& xyz, const u32arr& nn, const u32arr& nn_ptr, uint64_t k_min,
                    const std::vector<uint32_t>& k_scales, uint32_t k_step, uint32_t k_min_search, bool verbose) {
    const int64_t n_xyz = cloud_rows(xyz, "xyz");
    const int64_t nnz = vec_len(nn, "nn"), np1 = vec_len(nn_ptr, "nn_ptr");
    const int64_t n = np1 - 1, rows = std::max<int64_t>(n, 0);
    f64arr out = kind == 1 ? result_array<double>({rows, (int64_t)k_scales.size(), (int64_t)11})
                           : result_array<double>({rows, (int64_t)(kind == 2 ? 12 : 11)});
    int st;
    {
        py::gil_scoped_release nogil;
        if (kind == 0)
            st = pgeof_host_compute_features_f64(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n, k_min,
                                                 out.mutable_data());
        else if (kind == 1)
            st = pgeof_host_compute_features_multiscale_f64(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n,
                                                            k_scales.data(), (int64_t)k_scales.size(),
                                                            out.mutable_data());
        else
            st = pgeof_host_compute_features_optimal_f64(xyz.data(), n_xyz, nn.data(), nnz, nn_ptr.data(), n,
                                                         (uint32_t)k_min, k_step, k_min_search, out.mutable_data());
    }
    check(st);
    progress_done(verbose, n);
    return out;
}

std::pair<u32arr, f32arr> knn_search(const f32arr& data, const f32arr& query, uint32_t knn) {
    const int64_t n = cloud_rows(data, "data"), m = cloud_rows(query, "query");
    u32arr idx = result_array<uint32_t>({m, (int64_t)knn});
    f32arr d2 = result_array<float>({m, (int64_t)knn});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_knn_search_f32(data.data(), n, query.data(), m, knn, idx.mutable_data(), d2.mutable_data());
    }
    check(st);
    return {idx, d2};
}

std::pair<py::array_t<int32_t>, f32arr> radius_search(const f32arr& data, const f32arr& query, float search_radius,
                                                       uint32_t max_knn) {
    const int64_t n = cloud_rows(data, "data"), m = cloud_rows(query, "query");
    py::array_t<int32_t> idx = result_array<int32_t>({m, (int64_t)max_knn});
    f32arr d2 = result_array<float>({m, (int64_t)max_knn});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_radius_search_f32(data.data(), n, query.data(), m, search_radius, max_knn,
                                          idx.mutable_data(), d2.mutable_data());
    }
    check(st);
    return {idx, d2};
}

std::vector<int32_t> id_list(const std::vector<pgeof_feature_id>& ids) {
    std::vector<int32_t> v;
    v.reserve(ids.size());
    for (auto id : ids) v.push_back((int32_t)id);
    return v;
}

f64arr selected_f64(const f64arr& xyz, double search_radius, uint32_t max_knn,
                    const std::vector<pgeof_feature_id>& selected) {
    const int64_t n = cloud_rows(xyz, "xyz");
    const std::vector<int32_t> ids = id_list(selected);
    f64arr out = result_array<double>({n, (int64_t)ids.size()});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_compute_features_selected_f64(xyz.data(), n, search_radius, max_knn, ids.data(),
                                                      (int64_t)ids.size(), out.mutable_data());
    }
    check(st);
    return out;
}

f32arr selected_f32(const f32arr& xyz, float search_radius, uint32_t max_knn,
                    const std::vector<pgeof_feature_id>& selected) {
    const int64_t n = cloud_rows(xyz, "xyz");
    const std::vector<int32_t> ids = id_list(selected);
    f32arr out = result_array<float>({n, (int64_t)ids.size()});
    int st;
    {
        py::gil_scoped_release nogil;
        st = pgeof_host_compute_features_selected_f32(xyz.data(), n, search_radius, max_knn, ids.data(),
                                                      (int64_t)ids.size(), out.mutable_data());
    }
    check(st);
    return out;
}

// ------------------------------------------------------------------ device API
template <typename T>
T* P(uintptr_t p) {
    return reinterpret_cast<T*>(p);
}

}  // namespace

PYBIND11_MODULE(pgeof_ext, m) {
    m.doc() =
        "Compute, for each point in a 3D point cloud, local geometric features in parallel on a GB300 GPU "
        "(drop-in for pgeof's pgeof_ext)";

    py::enum_<pgeof_feature_id>(m, "EFeatureID")
        .value("Linearity", PGEOF_LINEARITY)
        .value("Planarity", PGEOF_PLANARITY)
        .value("Scattering", PGEOF_SCATTERING)
        .value("VerticalityPGEOF", PGEOF_VERTICALITY_PGEOF)
        .value("Normal_x", PGEOF_NORMAL_X)
        .value("Normal_y", PGEOF_NORMAL_Y)
        .value("Normal_z", PGEOF_NORMAL_Z)
        .value("Length", PGEOF_LENGTH)
        .value("Surface", PGEOF_SURFACE)
        .value("Volume", PGEOF_VOLUME)
        .value("Curvature", PGEOF_CURVATURE)
        .value("K_optimal", PGEOF_K_OPTIMAL)
        .value("Verticality", PGEOF_VERTICALITY)
        .value("Eigentropy", PGEOF_EIGENTROPY)
        .export_values();

    m.def("compute_features", &compute_features, py::arg("xyz").noconvert(), py::arg("nn").noconvert(),
          py::arg("nn_ptr").noconvert(), py::arg("k_min") = 1, py::arg("verbose") = false,
          "Compute the 11 geometric features of every point from a CSR neighbourhood (nn, nn_ptr).\n"
          "Rows with fewer than k_min neighbours are 0. Returns a (n_points, 11) float32 array.");
    m.def("compute_features_multiscale", &compute_features_multiscale, py::arg("xyz").noconvert(),
          py::arg("nn").noconvert(), py::arg("nn_ptr").noconvert(), py::arg("k_scales"), py::arg("verbose") = false,
          "Features at several neighbourhood sizes (prefixes of each CSR row); k_scales must be >= 1 and\n"
          "non-decreasing. Returns a (n_points, n_scales, 11) float32 array.");
    m.def("compute_features_optimal", &compute_features_optimal, py::arg("xyz").noconvert(),
          py::arg("nn").noconvert(), py::arg("nn_ptr").noconvert(), py::arg("k_min") = 1, py::arg("k_step") = 1,
          py::arg("k_min_search") = 1, py::arg("verbose") = false,
          "Features at the neighbourhood size of minimal eigentropy (Weinmann et al. 2015).\n"
          "Returns a (n_points, 12) float32 array; column 11 is the optimal size.");
    m.def(
        "compute_features_f64",
        [](const f64arr& xyz, const u32arr& nn, const u32arr& nn_ptr, uint64_t k_min, bool verbose) {
            return features_f64(0, xyz, nn, nn_ptr, k_min, {}, 1, 1, verbose);
        },
        py::arg("xyz").noconvert(), py::arg("nn").noconvert(), py::arg("nn_ptr").noconvert(), py::arg("k_min") = 1,
        py::arg("verbose") = false, "compute_features for a float64 cloud; (n_points, 11) float64.");
    m.def(
        "compute_features_multiscale_f64",
        [](const f64arr& xyz, const u32arr& nn, const u32arr& nn_ptr, const std::vector<uint32_t>& k_scales,
           bool verbose) { return features_f64(1, xyz, nn, nn_ptr, 1, k_scales, 1, 1, verbose); },
        py::arg("xyz").noconvert(), py::arg("nn").noconvert(), py::arg("nn_ptr").noconvert(), py::arg("k_scales"),
        py::arg("verbose") = false, "compute_features_multiscale for a float64 cloud; (n_points, n_scales, 11).");
    m.def(
        "compute_features_optimal_f64",
        [](const f64arr& xyz, const u32arr& nn, const u32arr& nn_ptr, uint32_t k_min, uint32_t k_step,
           uint32_t k_min_search, bool verbose) {
            return features_f64(2, xyz, nn, nn_ptr, k_min, {}, k_step, k_min_search, verbose);
        },
        py::arg("xyz").noconvert(), py::arg("nn").noconvert(), py::arg("nn_ptr").noconvert(), py::arg("k_min") = 1,
        py::arg("k_step") = 1, py::arg("k_min_search") = 1, py::arg("verbose") = false,
        "compute_features_optimal for a float64 cloud; (n_points, 12) float64, column 11 the optimal size.");
    m.def("knn_search", &knn_search, py::arg("data").noconvert(), py::arg("query").noconvert(), py::arg("knn"),
          "For each query point, the knn nearest data points: (uint32 indices, float32 squared distances),\n"
          "both (n_query, knn), ascending.");
    m.def("radius_search", &radius_search, py::arg("data").noconvert(), py::arg("query").noconvert(),
          py::arg("search_radius"), py::arg("max_knn"),
          "For each query point, up to max_knn nearest data points within search_radius: (int32 indices\n"
          "with -1 for missing, float32 squared distances with 0 for missing), both (n_query, max_knn).");
    m.def("compute_features_selected", &selected_f64, py::arg("xyz").noconvert(), py::arg("search_radius"),
          py::arg("max_knn"), py::arg("selected_features"),
          "Selected features from a radius neighbourhood (double precision version).");
    m.def("compute_features_selected", &selected_f32, py::arg("xyz").noconvert(), py::arg("search_radius"),
          py::arg("max_knn"), py::arg("selected_features"),
          "Selected features from a radius neighbourhood (float precision version).");

    // ---- library controls
    m.def("_abi_version", &pgeof_abi_version);
    m.def("_host_pool_trim", [] { check(pgeof_host_pool_trim()); });
    m.def("_launch_count", []() { return (uint64_t)pgeof_kernel_launch_count(); });
    m.def("_set_eig_order", [](int order) { check(pgeof_set_eig_order(order)); });
    m.def("_get_eig_order", &pgeof_get_eig_order);
    m.def("_profile_enable", [](bool on) { check(pgeof_profile_enable(on ? 1 : 0)); });
    m.def("_profile_report", []() {
        std::string buf(1 << 16, '\0');
        int st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_profile_report(&buf[0], buf.size());
        }
        check(st);
        buf.resize(strlen(buf.c_str()));
        return buf;
    });
    m.def("_take_device_errors", [](uintptr_t stream) {
        uint32_t bits = 0;
        int st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_take_device_errors(P<void>(stream), &bits);
        }
        check(st);
        return bits;
    });

    // ---- device-pointer entry points (raw pointers as integers)
    m.def("_dev_knn_search", [](uintptr_t data, int64_t n, uintptr_t query, int64_t m_, uint32_t k, uintptr_t idx,
                                uintptr_t d2, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_knn_search_f32(P<const float>(data), n, P<const float>(query), m_, k, P<uint32_t>(idx),
                                   P<float>(d2), P<void>(stream)));
    });
    m.def("_dev_radius_search", [](uintptr_t data, int64_t n, uintptr_t query, int64_t m_, float r, uint32_t k,
                                   uintptr_t idx, uintptr_t d2, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_radius_search_f32(P<const float>(data), n, P<const float>(query), m_, r, k, P<int32_t>(idx),
                                      P<float>(d2), P<void>(stream)));
    });
    m.def("_dev_radius_search_csr", [](uintptr_t data, int64_t n, uintptr_t query, int64_t m_, float r, uint32_t k,
                                       uintptr_t nn, uintptr_t nn_ptr, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_radius_search_csr_f32(P<const float>(data), n, P<const float>(query), m_, r, k, P<uint32_t>(nn),
                                          P<uint32_t>(nn_ptr), P<void>(stream)));
    });
    m.def("_dev_knn_features", [](uintptr_t xyz, int64_t n, uint32_t knn, std::vector<uint32_t> scales,
                                  uintptr_t out, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_knn_features_f32(P<const float>(xyz), n, knn, scales.data(), (int64_t)scales.size(),
                                     P<float>(out), P<void>(stream)));
    });
    m.def("_dev_compute_features", [](uintptr_t xyz, int64_t n_xyz, uintptr_t nn, int64_t nnz, uintptr_t ptr,
                                      int64_t n, uint64_t k_min, uintptr_t out, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_compute_features_f32(P<const float>(xyz), n_xyz, P<const uint32_t>(nn), nnz,
                                         P<const uint32_t>(ptr), n, k_min, P<float>(out), P<void>(stream)));
    });
    m.def("_dev_compute_features_multiscale",
          [](uintptr_t xyz, int64_t n_xyz, uintptr_t nn, int64_t nnz, uintptr_t ptr, int64_t n,
             const std::vector<uint32_t>& scales, uintptr_t out, uintptr_t stream) {
              py::gil_scoped_release nogil;
              check(pgeof_compute_features_multiscale_f32(P<const float>(xyz), n_xyz, P<const uint32_t>(nn), nnz,
                                                          P<const uint32_t>(ptr), n, scales.data(),
                                                          (int64_t)scales.size(), P<float>(out), P<void>(stream)));
          });
    m.def("_dev_compute_features_optimal",
          [](uintptr_t xyz, int64_t n_xyz, uintptr_t nn, int64_t nnz, uintptr_t ptr, int64_t n, uint32_t k_min,
             uint32_t k_step, uint32_t k_min_search, uintptr_t out, uintptr_t stream) {
              py::gil_scoped_release nogil;
              check(pgeof_compute_features_optimal_f32(P<const float>(xyz), n_xyz, P<const uint32_t>(nn), nnz,
                                                       P<const uint32_t>(ptr), n, k_min, k_step, k_min_search,
                                                       P<float>(out), P<void>(stream)));
          });
    m.def("_dev_batch_knn_features", [](uintptr_t xyz, const std::vector<int64_t>& offsets, uint32_t k, uintptr_t idx,
                                        uintptr_t d2, uintptr_t feats, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_batch_knn_features_f32(P<const float>(xyz), offsets.data(), (int64_t)offsets.size() - 1, k,
                                           P<uint32_t>(idx), P<float>(d2), P<float>(feats), P<void>(stream)));
    });
    m.def("_batch_plan_create", [](uintptr_t xyz, const std::vector<int64_t>& offsets, uint32_t k, uintptr_t idx,
                                   uintptr_t d2, uintptr_t feats, uintptr_t stream) {
        pgeof_batch_plan plan = nullptr;
        int st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_batch_plan_create(P<const float>(xyz), offsets.data(), (int64_t)offsets.size() - 1, k,
                                         P<uint32_t>(idx), P<float>(d2), P<float>(feats), P<void>(stream), &plan);
        }
        check(st);
        return reinterpret_cast<uintptr_t>(plan);
    });
    m.def("_batch_plan_launch", [](uintptr_t plan, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_batch_plan_launch(reinterpret_cast<pgeof_batch_plan>(plan), P<void>(stream)));
    });
    m.def("_batch_plan_info", [](uintptr_t plan) {
        float cell = 0.0f, tuned = 0.0f, dflt = 0.0f;
        uint32_t chunk = 0;
        int cached = 0;
        check(pgeof_batch_plan_info(reinterpret_cast<pgeof_batch_plan>(plan), &cell, &chunk, &tuned, &dflt, &cached));
        return py::make_tuple(cell, chunk, tuned, dflt, cached != 0);
    });
    m.def("_batch_plan_destroy", [](uintptr_t plan) {
        check(pgeof_batch_plan_destroy(reinterpret_cast<pgeof_batch_plan>(plan)));
    });
    m.def("_server_create", [](int slots, uint64_t budget) {
        pgeof_server sv = nullptr;
        check(pgeof_server_create(slots, budget, &sv));
        return reinterpret_cast<uintptr_t>(sv);
    });
    m.def("_server_submit", [](uintptr_t sv, uintptr_t xyz, int64_t n, double r, uint32_t max_knn,
                               const std::vector<int32_t>& ids, uintptr_t out, bool f64) {
        uint64_t id = 0;
        if (f64)
            check(pgeof_server_submit_selected_f64(reinterpret_cast<pgeof_server>(sv), P<const double>(xyz), n, r,
                                                   max_knn, ids.data(), (int64_t)ids.size(), P<double>(out), &id));
        else
            check(pgeof_server_submit_selected_f32(reinterpret_cast<pgeof_server>(sv), P<const float>(xyz), n,
                                                   (float)r, max_knn, ids.data(), (int64_t)ids.size(), P<float>(out),
                                                   &id));
        return id;
    });
    m.def("_server_add_cloud", [](uintptr_t sv, uintptr_t xyz, int64_t n, float radius_hint, uint32_t k_hint) {
        uint64_t cid = 0;
        int st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_server_add_cloud_f32(reinterpret_cast<pgeof_server>(sv), P<const float>(xyz), n, radius_hint,
                                            k_hint, &cid);
        }
        check(st);
        return cid;
    });
    m.def("_server_remove_cloud", [](uintptr_t sv, uint64_t cid) {
        py::gil_scoped_release nogil;
        check(pgeof_server_remove_cloud(reinterpret_cast<pgeof_server>(sv), cid));
    });
    m.def("_server_submit_resident", [](uintptr_t sv, uint64_t cid, double r, uint32_t max_knn,
                                        const std::vector<int32_t>& ids, uintptr_t out) {
        uint64_t id = 0;
        check(pgeof_server_submit_selected_resident_f32(reinterpret_cast<pgeof_server>(sv), cid, (float)r, max_knn,
                                                        ids.data(), (int64_t)ids.size(), P<float>(out), &id));
        return id;
    });
    m.def("_server_wait", [](uintptr_t sv, uint64_t id) {
        double lat = 0.0, qms = 0.0;
        int slot = -1, st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_server_wait(reinterpret_cast<pgeof_server>(sv), id, &lat, &qms, &slot);
        }
        check(st);
        return py::make_tuple(lat, qms, slot);
    });
    m.def("_server_stats", [](uintptr_t sv) {
        uint64_t peak = 0, done = 0;
        int peak_n = 0;
        check(pgeof_server_stats(reinterpret_cast<pgeof_server>(sv), &peak, &peak_n, &done));
        return py::make_tuple(peak, peak_n, done);
    });
    m.def("_server_destroy", [](uintptr_t sv) {
        py::gil_scoped_release nogil;
        check(pgeof_server_destroy(reinterpret_cast<pgeof_server>(sv)));
    });
    m.def("_index_create", [](uintptr_t data, int64_t n, uint32_t k_hint, float radius_hint, uintptr_t stream) {
        pgeof_index ix = nullptr;
        int st;
        {
            py::gil_scoped_release nogil;
            st = pgeof_index_create_f32(P<const float>(data), n, k_hint, radius_hint, P<void>(stream), &ix);
        }
        check(st);
        return reinterpret_cast<uintptr_t>(ix);
    });
    m.def("_index_destroy", [](uintptr_t ix) {
        py::gil_scoped_release nogil;
        check(pgeof_index_destroy(reinterpret_cast<pgeof_index>(ix)));
    });
    m.def("_dev_index_knn_search", [](uintptr_t ix, uintptr_t query, int64_t m_, uint32_t k, uintptr_t idx,
                                      uintptr_t d2, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_index_knn_search_f32(reinterpret_cast<pgeof_index>(ix), P<const float>(query), m_, k,
                                         P<uint32_t>(idx), P<float>(d2), P<void>(stream)));
    });
    m.def("_dev_index_radius_search", [](uintptr_t ix, uintptr_t query, int64_t m_, float r, uint32_t k,
                                         uintptr_t idx, uintptr_t d2, uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_index_radius_search_f32(reinterpret_cast<pgeof_index>(ix), P<const float>(query), m_, r, k,
                                            P<int32_t>(idx), P<float>(d2), P<void>(stream)));
    });
    m.def("_dev_index_knn_features", [](uintptr_t ix, uint32_t knn, std::vector<uint32_t> scales, uintptr_t out,
                                        uintptr_t stream) {
        py::gil_scoped_release nogil;
        check(pgeof_index_knn_features_f32(reinterpret_cast<pgeof_index>(ix), knn, scales.data(),
                                           (int64_t)scales.size(), P<float>(out), P<void>(stream)));
    });
    m.def("_dev_compute_features_f64",
          [](int kind, uintptr_t xyz, int64_t n_xyz, uintptr_t nn, int64_t nnz, uintptr_t ptr, int64_t n,
             uint64_t k_min, const std::vector<uint32_t>& scales, uint32_t k_step, uint32_t k_min_search,
             uintptr_t out, uintptr_t stream) {
              py::gil_scoped_release nogil;
              if (kind == 0)
                  check(pgeof_compute_features_f64(P<const double>(xyz), n_xyz, P<const uint32_t>(nn), nnz,
                                                   P<const uint32_t>(ptr), n, k_min, P<double>(out), P<void>(stream)));
              else if (kind == 1)
                  check(pgeof_compute_features_multiscale_f64(P<const double>(xyz), n_xyz, P<const uint32_t>(nn),
                                                              nnz, P<const uint32_t>(ptr), n, scales.data(),
                                                              (int64_t)scales.size(), P<double>(out),
                                                              P<void>(stream)));
              else
                  check(pgeof_compute_features_optimal_f64(P<const double>(xyz), n_xyz, P<const uint32_t>(nn), nnz,
                                                           P<const uint32_t>(ptr), n, (uint32_t)k_min, k_step,
                                                           k_min_search, P<double>(out), P<void>(stream)));
          });
    m.def("_dev_compute_features_selected",
          [](uintptr_t xyz, int64_t n, double r, uint32_t max_knn, const std::vector<int32_t>& ids, bool f64,
             uintptr_t out, uintptr_t stream) {
              py::gil_scoped_release nogil;
              if (f64)
                  check(pgeof_compute_features_selected_f64(P<const double>(xyz), n, r, max_knn, ids.data(),
                                                            (int64_t)ids.size(), P<double>(out), P<void>(stream)));
              else
                  check(pgeof_compute_features_selected_f32(P<const float>(xyz), n, (float)r, max_knn, ids.data(),
                                                            (int64_t)ids.size(), P<float>(out), P<void>(stream)));
          });
}
