// Internal state behind the C ABI handles.
#pragma once
#include <atomic>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "vh_common.cuh"
#include "vh_chol.cuh"
#include "vh_conv.cuh"

// Handles are reference counted: a geometry holds its context and a preconditioner its geometry,
// so the owner may destroy them in any order; a parent is released with its last child.
struct vh_precon;

struct vh_ctx {
  std::atomic<int> refs{1};
  int device = 0;
  cudaStream_t stream = nullptr;
  std::string last_error;
  vh::Profiler prof;
  vh::DevicePool pool;   // solver buffers and factors; all their work is ordered on `stream`
};

namespace vh {

// Real CSR matrix on the device.
struct Csr {
  int64_t nrows = 0, ncols = 0, nnz = 0;
  int32_t* rowptr = nullptr;  // nrows + 1 (nnz < 2^31 checked)
  int32_t* col = nullptr;
  double* val = nullptr;
  void free_all() {
    cudaFree(rowptr);
    cudaFree(col);
    cudaFree(val);
    rowptr = nullptr; col = nullptr; val = nullptr;
  }
};

// y[b*ldy + yoff + r] (mode 0: =, 1: +=, -1: -=) sum_j A(r, j) x[b*ldx + xoff + j]
void spmv_batched(const Csr& A, int B, const double2* x, int64_t ldx, int64_t xoff, double2* y, int64_t ldy,
                  int64_t yoff, int mode, cudaStream_t st);

// Host copy of a CSR matrix.
struct HostCsr {
  std::vector<int32_t> rp, col;
  std::vector<double> val;
};

// Host CSC (nrow x ncol) -> host CSR of A and of A^T.
void csc_to_host(int64_t nrow, int64_t ncol, const int64_t* jc, const int64_t* ir, const double* pr, HostCsr& hA,
                 HostCsr& hAT);

// Host CSC (num_node x ncol) -> device CSR of A and of A^T (host copies returned too).
void csc_upload(int64_t nrow, int64_t ncol, const int64_t* jc, const int64_t* ir, const double* pr, Csr& A, Csr& AT,
                HostCsr& hA, HostCsr& hAT, cudaStream_t st);

}  // namespace vh

struct vh_geom {
  std::atomic<int> refs{1};
  vh_ctx* ctx = nullptr;
  int L = 0, M = 0, N = 0;
  double dx = 0;
  int64_t nv = 0, nc = 0, nphi = 0, n = 0;
  std::vector<int64_t> idxS;       // host copy, 1-based
  vh::ConvPlan conv;
  vh::Csr Ae, AeT;                 // nphi x nc, nc x nphi
  vh::HostCsr hAe, hAeT;           // host copies (symbolic analysis)
  bool has_conv = false;           // false for a preconditioner-only geometry (no tensor)
  vh::CholSymbolic chol;           // built on the first 'schur_invert' preconditioner
  bool chol_ready = false;
  double2* pc_tmp = nullptr;       // chol_solve update vectors, B * u_total (16-byte complex values)
  void* pc_phi_df = nullptr;       // double-float factor: B * nphi pair-complex panel values being solved
  double* approx_w = nullptr;      // 'schur_approx': 1 / sum_k |Ae(r, k)| per panel row r (device)
  size_t pc_phi_df_cap = 0;
  size_t pc_tmp_cap = 0;
  double** pc_ptrs = nullptr;      // device pointer tables (A_inv, W) for batched applies
  int pc_ptrs_cap = 0;
  std::vector<double2*> zslots;    // per slot: nv complex (device)
  double2* ones = nullptr;         // device, capacity ones_cap complex ones
  int ones_cap = 0;
  double2* io_x = nullptr;         // staging for host-pointer calls
  double2* io_y = nullptr;
  double2* io_s = nullptr;
  size_t io_cap = 0;               // RHS capacity of io_x / io_y
  double2* zgather = nullptr;      // B x nv gathered z for mixed slots
  size_t zgather_cap = 0;
};

namespace vh {
// Drop one reference; the last one frees the handle (and releases its parent).
void ctx_release(vh_ctx* c);
void geom_release(vh_geom* g);
}  // namespace vh

namespace vh {
struct GmresOut {
  std::vector<int> flag, inner, outer;
  std::vector<double> relres;
  std::vector<std::vector<double>> resvec;
  int64_t matvecs = 0;   // RHS-matvecs performed
  int64_t precons = 0;
};

// A batch of linear operators for the Krylov solver: A and M act on the rows `act` of the batch
// (x, y compact: row a of x belongs to RHS act[a]); M empty = no preconditioner.  All work is
// ordered on `st`.
struct KrylovOps {
  int64_t n = 0;
  cudaStream_t st = nullptr;
  Profiler* prof = nullptr;   // Krylov vector work is timed here (nullptr: not timed)
  std::function<void(const std::vector<int>& act, const double2* x, double2* y, Prec p)> A;
  std::function<void(const std::vector<int>& act, const double2* x, double2* y)> M;
};

// Restarted left-preconditioned GMRES (pgmres.m semantics) or flexible GMRES (fpgmres.m), batched.
void gmres_core(const KrylovOps& op, int B, const double2* b, const double* tol, int m, int maxit, bool flexible,
                Prec prec, double2* x, GmresOut& out, bool true_relres, const double2* pre_Mb);

// Inner GMRES on the Schur complements of the 'schur_gmres' preconditioner (Jacobi-preconditioned).
void schur_gmres_solve(vh_geom* g, int B, double* const* ainv, double* const* sdiag, const double2* bb, double2* phi,
                       int64_t ldphi, const double* tol, int restart, int maxit, int* iters);

// The kind (vh_precon_kind) of a preconditioner handle.
int precon_kind(const vh_precon* p);
}  // namespace vh
