// PyTorch extension module `pamo_gb300._C`: the reference's operator module `pamo._C` (simp_cuda/src/pybind.cpp) with
// the same class names, constructor and forward() signatures, over the C ABI of include/pamo_gb300.h. Tensors are
// plumbing only: every call goes to libpamo_gb300.so (hand-written sm_103a kernels) on the tensor's device and the
// current torch stream; outputs are new tensors, as the reference's clone()s are.
//
//   CUDSP_Free().forward(points f32[N,3], triangles i32[M,3], verts_undo i32[K], n_verts_undo, scale, threshold,
//                        is_stuck, init) -> (verts, tris, verts_occ, verts_map, verts_undo)      pybind.cpp:52-103
//   CUDSP().forward(points, triangles, scale, threshold, init) -> (verts, tris, verts_occ, verts_map)
//                                                                                                pybind.cpp:140-182
// Input checks raise like the reference's CHECK_INPUT / TORCH_INTERNAL_ASSERT (pybind.cpp:8-14, 59-63); a failed
// call raises with the library's status message (the reference prints CUDA errors and goes on).
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>
#include <torch/extension.h>

#include "../../include/pamo_gb300.h"

namespace {

void check_input(const at::Tensor& t, const char* name) {
    TORCH_CHECK(t.is_cuda(), name, " must be a CUDA tensor");
    TORCH_CHECK(t.is_contiguous(), name, " must be contiguous");
}

// one pamo_ctx per operator instance and device, created on first use like the reference's lazily grown buffers
struct Operator {
    pamo_ctx* ctx = nullptr;
    int device = -1;
    Operator() = default;
    Operator(const Operator&) = delete;
    Operator& operator=(const Operator&) = delete;
    ~Operator() {
        if (ctx) pamo_ctx_destroy(ctx);
    }
    pamo_ctx* on(int dev) {
        if (ctx && device != dev) {
            pamo_ctx_destroy(ctx);
            ctx = nullptr;
        }
        if (!ctx) {
            const int rc = pamo_ctx_create(&ctx, dev);
            TORCH_CHECK(rc == PAMO_OK, "pamo_ctx_create: ", pamo_status_string(rc));
            device = dev;
        }
        return ctx;
    }
    void check(int rc) const {
        TORCH_CHECK(rc == PAMO_OK, "pamo: ", pamo_status_string(rc), ": ", ctx ? pamo_ctx_last_error(ctx) : "");
    }
};

struct CUDSP_Free : Operator {
    std::tuple<at::Tensor, at::Tensor, at::Tensor, at::Tensor, at::Tensor> forward(
        at::Tensor points, at::Tensor triangles, at::Tensor verts_undo, int64_t n_verts_undo, double scale,
        double threshold, bool is_stuck, bool init) {
        check_input(points, "points");
        check_input(triangles, "triangles");
        check_input(verts_undo, "verts_undo");
        TORCH_CHECK(points.scalar_type() == at::kFloat, "points type must match the pamo class");
        TORCH_CHECK(triangles.scalar_type() == at::kInt, "triangles type must match the pamo class");
        TORCH_CHECK(verts_undo.scalar_type() == at::kInt, "verts_undo must be int32");
        const c10::cuda::CUDAGuard guard(points.device());
        pamo_ctx* c = on(points.get_device());
        cudaStream_t s = c10::cuda::getCurrentCUDAStream(points.get_device()).stream();
        check(pamo_forward_round(c, points.data_ptr<float>(), triangles.data_ptr<int32_t>(),
                                 verts_undo.numel() ? verts_undo.data_ptr<int32_t>() : nullptr, (int32_t)n_verts_undo,
                                 (int32_t)points.size(0), (int32_t)triangles.size(0), (float)scale, (float)threshold,
                                 is_stuck ? 1 : 0, init ? 1 : 0, s));
        int32_t np = 0, nt = 0, nu = 0;
        check(pamo_round_sizes(c, &np, &nt, &nu));
        const auto of = points.options();
        const auto oi = triangles.options();
        at::Tensor v = at::empty({np, 3}, of), f = at::empty({nt, 3}, oi), occ = at::empty({np, 1}, oi),
                   map = at::empty({np, 1}, oi), u = at::empty({nu}, oi);
        check(pamo_round_outputs(c, v.data_ptr<float>(), f.data_ptr<int32_t>(), occ.data_ptr<int32_t>(),
                                 map.data_ptr<int32_t>(), nu ? u.data_ptr<int32_t>() : nullptr, s));
        return {v, f, occ, map, u};
    }
};

struct CUDSP : Operator {
    std::tuple<at::Tensor, at::Tensor, at::Tensor, at::Tensor> forward(at::Tensor points, at::Tensor triangles,
                                                                       double scale, double threshold, bool init) {
        check_input(points, "points");
        check_input(triangles, "triangles");
        TORCH_CHECK(points.scalar_type() == at::kFloat, "points type must match the sp class");
        TORCH_CHECK(triangles.scalar_type() == at::kInt, "triangles type must match the sp class");
        const c10::cuda::CUDAGuard guard(points.device());
        pamo_ctx* c = on(points.get_device());
        cudaStream_t s = c10::cuda::getCurrentCUDAStream(points.get_device()).stream();
        check(pamo_legacy_round(c, points.data_ptr<float>(), triangles.data_ptr<int32_t>(), (int32_t)points.size(0),
                                (int32_t)triangles.size(0), (float)scale, (float)threshold, init ? 1 : 0, s));
        int32_t np = 0, nt = 0, nu = 0;
        check(pamo_round_sizes(c, &np, &nt, &nu));
        const auto oi = triangles.options();
        at::Tensor v = at::empty({np, 3}, points.options()), f = at::empty({nt, 3}, oi), occ = at::empty({np, 1}, oi),
                   map = at::empty({np, 1}, oi);
        check(pamo_round_outputs(c, v.data_ptr<float>(), f.data_ptr<int32_t>(), occ.data_ptr<int32_t>(),
                                 map.data_ptr<int32_t>(), nullptr, s));
        return {v, f, occ, map};
    }
};

}  // namespace

PYBIND11_MODULE(_C, m) {
    m.doc() = "pamo._C over the pamo_gb300 C ABI (sm_103a kernels)";
    pybind11::class_<CUDSP_Free>(m, "CUDSP_Free")
        .def(pybind11::init<>())
        .def("forward", &CUDSP_Free::forward, pybind11::arg("points"), pybind11::arg("triangles"),
             pybind11::arg("verts_undo"), pybind11::arg("n_verts_undo"), pybind11::arg("scale"),
             pybind11::arg("threshold"), pybind11::arg("is_stuck"), pybind11::arg("init"));
    pybind11::class_<CUDSP>(m, "CUDSP")
        .def(pybind11::init<>())
        .def("forward", &CUDSP::forward, pybind11::arg("points"), pybind11::arg("triangles"), pybind11::arg("scale"),
             pybind11::arg("threshold"), pybind11::arg("init"));
}
