// PyTorch C++ extension named `spmm`: the GCN custom op of the reference
// (gcn/pytorch-custom/spmm.cpp:95-114, bound at :167-172) on CUDA tensors, plus the SDDMM
// and CSR->CSC ops its sibling files declare (sddmm.cpp:21-61, spmm_kernel.cu:460-476).
// Every op checks its tensors with TORCH_CHECK (the reference used assert, compiled out
// under NDEBUG), runs on the current CUDA stream through the C ABI (armsparse_gpu.h), and
// zero-initialises nothing it overwrites: csr_spmm writes every output element (the
// reference's torch::empty + "+=" read uninitialised memory, spmm.cpp:41).
#include <torch/extension.h>
#include <c10/cuda/CUDAGuard.h>
#include <c10/cuda/CUDAStream.h>

#include <cuda_runtime.h>

#include <mutex>
#include <unordered_map>

#include "armsparse_gpu.h"

namespace {

as_ctx *ctx_for(int device) {
    thread_local std::unordered_map<int, as_ctx *> ctxs;
    auto it = ctxs.find(device);
    if (it != ctxs.end()) return it->second;
    as_ctx *c = nullptr;
    as_status st = as_ctx_create(&c, device);
    TORCH_CHECK(st == AS_OK, "armsparse: context creation failed: ", as_last_error());
    ctxs[device] = c;
    return c;
}

// the current torch stream of the tensor's device
void *stream_of(const torch::Tensor &t) {
    return reinterpret_cast<void *>(c10::cuda::getCurrentCUDAStream(t.device().index()).stream());
}

void check(as_status st, const char *what) {
    TORCH_CHECK(st == AS_OK, what, ": ", as_status_string(st), ": ", as_last_error());
}

void need(const torch::Tensor &t, const char *name, c10::ScalarType dt, int dim) {
    TORCH_CHECK(t.is_cuda(), name, " must be a CUDA tensor (there is no CPU path)");
    TORCH_CHECK(t.is_contiguous(), name, " must be contiguous");
    TORCH_CHECK(t.scalar_type() == dt, name, " has the wrong dtype");
    TORCH_CHECK(t.dim() == dim, name, " must have ", dim, " dims");
}

}  // namespace

// out = A * dense, A (m x k) in CSR; dense (k x n). fp32 or bf16 (values and dense in the
// same dtype; output fp32).
torch::Tensor csr_spmm(torch::Tensor rowptr, torch::Tensor colind, torch::Tensor values,
                       torch::Tensor dense) {
    need(rowptr, "rowptr", torch::kInt32, 1);
    need(colind, "colind", torch::kInt32, 1);
    TORCH_CHECK(dense.is_cuda() && dense.is_contiguous() && dense.dim() == 2,
                "dense must be a contiguous 2-D CUDA tensor");
    TORCH_CHECK(values.scalar_type() == dense.scalar_type(), "values and dense dtypes differ");
    need(values, "values", dense.scalar_type(), 1);
    TORCH_CHECK(values.numel() == colind.numel(), "values and colind lengths differ");
    const int m = static_cast<int>(rowptr.size(0) - 1);
    const int k = static_cast<int>(dense.size(0));
    const int n = static_cast<int>(dense.size(1));
    const int nnz = static_cast<int>(colind.numel());
    c10::cuda::CUDAGuard g(dense.device());
    auto out = torch::empty({m, n}, dense.options().dtype(torch::kFloat32));
    as_ctx *c = ctx_for(dense.device().index());
    if (dense.scalar_type() == torch::kFloat32) {
        check(as_spmm_csr_f32(c, m, k, n, nnz, rowptr.data_ptr<int>(), colind.data_ptr<int>(),
                              values.data_ptr<float>(), dense.data_ptr<float>(), n,
                              out.data_ptr<float>(), n, 0.0f, 0, stream_of(dense)),
              "csr_spmm");
    } else {
        TORCH_CHECK(dense.scalar_type() == torch::kBFloat16, "dense must be float32 or bfloat16");
        check(as_spmm_csr_bf16(c, m, k, n, nnz, rowptr.data_ptr<int>(), colind.data_ptr<int>(),
                               reinterpret_cast<const uint16_t *>(values.data_ptr()),
                               reinterpret_cast<const uint16_t *>(dense.data_ptr()), n,
                               out.data_ptr<float>(), n, 0.0f, 0, stream_of(dense)),
              "csr_spmm (bf16)");
    }
    return out;
}

// out[e] = <D1[row(e)], D2[col(e)]> in CSR order (sddmm.cu:459-483 semantics), optionally
// scaled by values; tensor_cores selects the split-bf16 tcgen05 path.
torch::Tensor csr_sddmm(torch::Tensor rowptr, torch::Tensor colind, torch::Tensor D1,
                        torch::Tensor D2, c10::optional<torch::Tensor> values, bool tensor_cores) {
    need(rowptr, "rowptr", torch::kInt32, 1);
    need(colind, "colind", torch::kInt32, 1);
    need(D1, "D1", torch::kFloat32, 2);
    need(D2, "D2", torch::kFloat32, 2);
    TORCH_CHECK(D1.size(1) == D2.size(1), "D1 and D2 need the same K");
    TORCH_CHECK(D1.size(0) == rowptr.size(0) - 1, "D1 needs one row per pattern row");
    const float *av = nullptr;
    if (values.has_value()) {
        need(*values, "values", torch::kFloat32, 1);
        av = values->data_ptr<float>();
    }
    const int m = static_cast<int>(rowptr.size(0) - 1);
    const int nnz = static_cast<int>(colind.numel());
    const int k = static_cast<int>(D1.size(1));
    c10::cuda::CUDAGuard g(D1.device());
    auto out = torch::empty({nnz}, D1.options());
    as_ctx *c = ctx_for(D1.device().index());
    auto fn = tensor_cores ? as_sddmm_csr_bf16x3 : as_sddmm_csr_f32;
    check(fn(c, m, static_cast<int>(D2.size(0)), k, nnz, rowptr.data_ptr<int>(),
             colind.data_ptr<int>(), av, D1.data_ptr<float>(), k, D2.data_ptr<float>(), k,
             out.data_ptr<float>(), stream_of(D1)),
          "csr_sddmm");
    return out;
}

// COO form (sddmm.cpp:21-40): out[e] = <D1[rowind[e]], D2[colind[e]]>, entries in any order.
torch::Tensor coo_sddmm(torch::Tensor rowind, torch::Tensor colind, torch::Tensor D1,
                        torch::Tensor D2) {
    need(rowind, "rowind", torch::kInt32, 1);
    need(colind, "colind", torch::kInt32, 1);
    need(D1, "D1", torch::kFloat32, 2);
    need(D2, "D2", torch::kFloat32, 2);
    TORCH_CHECK(rowind.numel() == colind.numel(), "rowind and colind lengths differ");
    TORCH_CHECK(D1.size(1) == D2.size(1), "D1 and D2 need the same K");
    const int nnz = static_cast<int>(colind.numel());
    const int k = static_cast<int>(D1.size(1));
    c10::cuda::CUDAGuard g(D1.device());
    auto out = torch::empty({nnz}, D1.options());
    check(as_sddmm_coo_f32(ctx_for(D1.device().index()), static_cast<int>(D1.size(0)),
                           static_cast<int>(D2.size(0)), k, nnz, rowind.data_ptr<int>(),
                           colind.data_ptr<int>(), nullptr, D1.data_ptr<float>(), k,
                           D2.data_ptr<float>(), k, out.data_ptr<float>(), stream_of(D1)),
          "coo_sddmm");
    return out;
}

// csr2csc(rowptr, colind, colptr, rowind, csr_data) -> csc_data; colptr (n+1) and rowind (nnz)
// are written in place (the argument order of the reference's commented binding,
// spmm.cpp:142-165, and csr2csc_cuda, spmm_kernel.cu:460-476). Rows ascend within columns.
torch::Tensor csr2csc(torch::Tensor rowptr, torch::Tensor colind, torch::Tensor colptr,
                      torch::Tensor rowind, torch::Tensor csr_data) {
    need(rowptr, "rowptr", torch::kInt32, 1);
    need(colind, "colind", torch::kInt32, 1);
    need(colptr, "colptr", torch::kInt32, 1);
    need(rowind, "rowind", torch::kInt32, 1);
    need(csr_data, "csr_data", torch::kFloat32, 1);
    const int m = static_cast<int>(rowptr.size(0) - 1);
    const int n = static_cast<int>(colptr.size(0) - 1);
    const int nnz = static_cast<int>(colind.numel());
    TORCH_CHECK(rowind.numel() == nnz && csr_data.numel() == nnz, "length mismatch");
    c10::cuda::CUDAGuard g(rowptr.device());
    auto cscval = torch::empty({nnz}, csr_data.options());
    check(as_csr2csc(ctx_for(rowptr.device().index()), m, n, nnz, rowptr.data_ptr<int>(),
                     colind.data_ptr<int>(), csr_data.data_ptr<float>(), colptr.data_ptr<int>(),
                     rowind.data_ptr<int>(), cscval.data_ptr<float>(), stream_of(rowptr)),
          "csr2csc");
    return cscval;
}

PYBIND11_MODULE(TORCH_EXTENSION_NAME, m) {
    m.doc() = "CSR SpMM, SDDMM and CSR->CSC on sm_103a (drop-in for the GCN op module `spmm`)";
    m.def("csr_spmm", &csr_spmm, "CSR SpMM: out = A * dense", py::arg("rowptr"),
          py::arg("colind"), py::arg("values"), py::arg("dense"));
    m.def("csr_sddmm", &csr_sddmm, "CSR SDDMM", py::arg("rowptr"), py::arg("colind"),
          py::arg("D1"), py::arg("D2"), py::arg("values") = py::none(),
          py::arg("tensor_cores") = false);
    m.def("coo_sddmm", &coo_sddmm, "COO SDDMM", py::arg("rowind"), py::arg("colind"),
          py::arg("D1"), py::arg("D2"));
    m.def("csr2csc", &csr2csc, "CSR -> CSC (colptr, rowind filled in place; returns values)",
          py::arg("rowptr"), py::arg("colind"), py::arg("colptr"), py::arg("rowind"),
          py::arg("csr_data"));
}
