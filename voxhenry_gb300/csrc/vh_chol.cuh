// Sparse Cholesky of the Schur complement S = Ar diag(A_inv) Ar^T (nphi x nphi, SPD) used by the
// 'schur_invert' preconditioner (lse_sparse_precon_prepare.m:90-191, lse_sparse_precon_multiply.m:61-117).
//
// Symbolic analysis (host, once per geometry): geometric nested dissection of the panel graph, a
// front per dissection node, row structures, extend-add maps and assembly term lists.
// Numeric factorisation (device, per frequency): multifrontal, level by level from the leaves.
// Solves (device): forward pass from the leaves with per-front update vectors, backward pass
// from the root.  The factor is real; right-hand sides are complex.
#pragma once
#include <vector>

#include "vh_common.cuh"

namespace vh {

// Fronts of at most this order are factored by one CTA with the whole front in shared memory.
constexpr int kFusedMaxNf = 160;

struct FrontInfo {
  int32_t ns;          // pivots (own panels)
  int32_t nb;          // boundary rows
  int32_t nf;          // ns + nb
  int32_t parent;      // -1 for a root
  int32_t child[2];    // -1 if absent
  int64_t w_off;       // dense nf x nf column-major front in the factor storage
  int64_t rows_off;    // rows[rows_off .. + nf): global panel index (own first)
  int64_t relmap_off;  // relmap[relmap_off .. + nb): local row in the parent for each boundary row
  int64_t asm_off;     // assembly entries [asm_off, asm_off + asm_cnt)
  int32_t asm_cnt;
  int32_t pad_;
  int64_t u_off;       // per-RHS update vector offset (nb entries)
};

struct AsmEntry {
  int32_t li, lj;      // local row / column (li >= lj, lj < ns)
  int32_t t0, t1;      // terms [t0, t1) in asm_q / asm_c
};

struct CholSymbolic {
  int64_t n = 0;                    // nphi
  int nfronts = 0;
  int max_nf = 0;
  int64_t w_total = 0;              // doubles of factor storage (sum nf^2)
  int64_t u_total = 0;              // sum nb (update vector length per RHS)
  int64_t nnz_l = 0;                // entries of L (sum over fronts of ns*(ns+1)/2 + nb*ns)
  double flops = 0;                 // factorisation flops
  std::vector<FrontInfo> fronts;
  std::vector<std::vector<int32_t>> levels;  // fronts per height (leaves first)
  std::vector<int32_t> level_max_ns, level_max_nf;
  // per height, the fronts factored whole in shared memory (nf <= kFusedMaxNf) and the others.
  // levels_fused[h] is sorted by decreasing order; fused_classes[h] cuts it into runs whose shared
  // memory lets the same number of CTAs share an SM, so that small fronts run at high occupancy.
  struct FusedClass {
    int32_t offset, count, max_nf, max_ns;
  };
  std::vector<std::vector<int32_t>> levels_fused, levels_blocked;
  std::vector<std::vector<FusedClass>> fused_classes;
  std::vector<int32_t> fused_max_ns, fused_max_nf, blocked_max_ns, blocked_max_nf;
  // device copies
  FrontInfo* d_fronts = nullptr;
  int32_t* d_rows = nullptr;
  int32_t* d_relmap = nullptr;
  AsmEntry* d_asm = nullptr;
  int32_t* d_asm_q = nullptr;
  double* d_asm_c = nullptr;
  std::vector<int32_t*> d_levels;   // per height: front ids
  std::vector<int32_t*> d_levels_fused, d_levels_blocked;
  int* d_err = nullptr;             // factorisation status flag
  mutable void** d_tab = nullptr;   // device pointer table of the batched factorisation
  mutable int tab_cap = 0;
  // side streams of the factorisation: the occupancy classes and the blocked fronts of one level
  // are independent and run concurrently, joined before the next level (created on first use)
  static constexpr int kSideStreams = 3;
  mutable cudaStream_t side[kSideStreams] = {};
  mutable cudaEvent_t ev_fork = nullptr;
  mutable cudaEvent_t ev_join[kSideStreams] = {};
  int64_t n_asm = 0;
  void free_all();
};

// Builds the symbolic structure from the host CSR of Ar (nphi x nc) and of Ar^T (nc x nphi),
// and the voxel linear indices (1-based) of the nv voxels.  Throws ERR_UNSUPPORTED when Ar does
// not have the VoxHenry incidence structure.
void chol_symbolic(CholSymbolic& s, int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t nphi,
                   const std::vector<int32_t>& a_rp, const std::vector<int32_t>& a_col, const std::vector<double>& a_val,
                   const std::vector<int32_t>& t_rp, const std::vector<int32_t>& t_col, const std::vector<double>& t_val,
                   int leaf_size, cudaStream_t st, bool to_device = true);

// Numeric factorisation of `nfac` factors at once (one per frequency): factor i goes to W[i]
// (sym.w_total values of T, device) from the diagonal D[i] = A_inv (nc doubles, device).  The
// pointer arrays are host arrays.  T = double, or dfloat (FP32 pairs) for the mixed-precision solver.
template <typename T>
void chol_factor(const CholSymbolic& s, int nfac, const double* const* D, T* const* W, cudaStream_t st);

// Solves S x = b in place for B right-hand sides in the factor's precision.  x: device, complex of
// T, RHS b at x + b*ldx + xoff (panel indexing); Wp: device array of B factor pointers; U: device
// scratch of B * u_total complex values of T.  xd (optional): the solution is also written there
// in complex128, RHS b at xd + b*ldxd (panel indexing).
template <typename T>
void chol_solve(const CholSymbolic& s, int B, T* const* Wp, cplx<T>* x, int64_t ldx, int64_t xoff, cplx<T>* U,
                cudaStream_t st, double2* xd = nullptr, int64_t ldxd = 0);

}  // namespace vh
