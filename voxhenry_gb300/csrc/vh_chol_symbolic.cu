// Symbolic analysis of the Schur complement S = Ar D Ar^T: geometric nested dissection of the
// panel graph and multifrontal structure.  Host code, run once per geometry.
//
// Panel geometry is recovered from Ar itself: the row of an x-panel holds the Jx entries of the
// (at most two) voxels it bounds, -1 on the voxel whose -x face it is and +1 on the voxel whose
// +x face it is (lse_compute_Ae_matrix.m:205-211); likewise y / z.  In doubled coordinates a
// panel on face f of axis a sits at 2f along a and at 2c+1 (voxel centre) along the others.  A
// cut at the face plane 2f along a separates the panels with coordinate < 2f from those > 2f:
// no voxel touches both sides, so the panels on the plane form a separator of S's graph.
#include <algorithm>
#include <cstring>
#include <functional>
#include <numeric>

#include "vh_chol.cuh"

namespace vh {

void CholSymbolic::free_all() {
  cudaFree(d_fronts);
  cudaFree(d_rows);
  cudaFree(d_relmap);
  cudaFree(d_asm);
  cudaFree(d_asm_q);
  cudaFree(d_asm_c);
  for (auto* p : d_levels) cudaFree(p);
  for (auto* p : d_levels_fused) cudaFree(p);
  for (auto* p : d_levels_blocked) cudaFree(p);
  d_levels_fused.clear();
  d_levels_blocked.clear();
  cudaFree(d_err);
  d_err = nullptr;
  cudaFree(d_tab);
  d_tab = nullptr;
  tab_cap = 0;
  for (int i = 0; i < kSideStreams; ++i) {
    if (side[i]) cudaStreamDestroy(side[i]);
    if (ev_join[i]) cudaEventDestroy(ev_join[i]);
    side[i] = nullptr;
    ev_join[i] = nullptr;
  }
  if (ev_fork) cudaEventDestroy(ev_fork);
  ev_fork = nullptr;
  d_levels.clear();
  d_fronts = nullptr; d_rows = nullptr; d_relmap = nullptr; d_asm = nullptr; d_asm_q = nullptr; d_asm_c = nullptr;
}

namespace {

struct Node {
  std::vector<int32_t> own;
  int child[2] = {-1, -1};
  int parent = -1;
};

template <typename T>
void upload(T*& dst, const std::vector<T>& src, cudaStream_t st) {
  const size_t bytes = std::max<size_t>(1, src.size()) * sizeof(T);
  VH_CUDA_TRY(cudaMalloc(&dst, bytes));
  if (!src.empty()) VH_CUDA_TRY(cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st));
}

}  // namespace

void chol_symbolic(CholSymbolic& s, int L, int M, int N, int64_t nv, const int64_t* idxS, int64_t nphi,
                   const std::vector<int32_t>& a_rp, const std::vector<int32_t>& a_col, const std::vector<double>& a_val,
                   const std::vector<int32_t>& t_rp, const std::vector<int32_t>& t_col, const std::vector<double>& t_val,
                   int leaf_size, cudaStream_t st, bool to_device) {
  s.n = nphi;
  // ---- panel coordinates (doubled)
  std::vector<int32_t> pc(3 * nphi);
  for (int64_t i = 0; i < nphi; ++i) {
    int found = -1;
    for (int32_t k = a_rp[i]; k < a_rp[i + 1]; ++k) {
      const int64_t q = a_col[k];
      const int c = (int)(q / nv);
      if (c <= 2 && (a_val[k] == 1.0 || a_val[k] == -1.0)) { found = k; break; }
    }
    VH_REQUIRE(found >= 0, ERR_UNSUPPORTED, "Ae row without a Jx/Jy/Jz entry: not a VoxHenry incidence matrix");
    const int64_t q = a_col[found];
    const int axis = (int)(q / nv);
    const int64_t v = q % nv;
    const int64_t li = idxS[v] - 1;
    int64_t co[3] = {li % L, (li / L) % M, li / ((int64_t)L * M)};
    for (int d = 0; d < 3; ++d) pc[3 * i + d] = (int32_t)(2 * co[d] + 1);
    pc[3 * i + axis] = (int32_t)(2 * (co[axis] + (a_val[found] > 0 ? 1 : 0)));
  }
  // ---- nested dissection
  std::vector<Node> nodes;
  std::function<int(std::vector<int32_t>&)> dissect = [&](std::vector<int32_t>& pan) -> int {
    const int id = (int)nodes.size();
    nodes.emplace_back();
    if ((int64_t)pan.size() <= leaf_size) {
      nodes[id].own = pan;
      return id;
    }
    int32_t lo[3] = {INT32_MAX, INT32_MAX, INT32_MAX}, hi[3] = {INT32_MIN, INT32_MIN, INT32_MIN};
    for (int32_t p : pan)
      for (int d = 0; d < 3; ++d) { lo[d] = std::min(lo[d], pc[3 * p + d]); hi[d] = std::max(hi[d], pc[3 * p + d]); }
    // Cut plane: over the three axes, the face plane (even coordinate) with the fewest panels on
    // it among those leaving at least a fraction `beta` of the panels on either side; beta is
    // relaxed when no plane qualifies.  Ties go to the better balanced plane.
    const int64_t n = (int64_t)pan.size();
    int best_a = -1;
    int32_t best_m = 0;
    for (double beta : {0.30, 0.15, 0.02}) {
      int64_t best_sep = INT64_MAX, best_imb = INT64_MAX;
      for (int a = 0; a < 3; ++a) {
        if (hi[a] - lo[a] < 2) continue;
        const int range = hi[a] - lo[a] + 1;
        std::vector<int64_t> cnt(range, 0);
        for (int32_t p : pan) cnt[pc[3 * p + a] - lo[a]]++;
        int64_t left = 0;
        for (int c = 0; c < range; ++c) {
          const int32_t m = lo[a] + c;
          if ((m & 1) == 0 && m > lo[a] && m < hi[a]) {
            const int64_t sep = cnt[c], right = n - left - sep;
            if (left >= beta * n && right >= beta * n && left > 0 && right > 0) {
              const int64_t imb = left > right ? left - right : right - left;
              if (sep < best_sep || (sep == best_sep && imb < best_imb)) {
                best_sep = sep;
                best_imb = imb;
                best_a = a;
                best_m = m;
              }
            }
          }
          left += cnt[c];
        }
      }
      if (best_a >= 0) break;
    }
    if (best_a >= 0) {
      const int a = best_a;
      const int32_t m = best_m;
      std::vector<int32_t> left, right, sep;
      for (int32_t p : pan) {
        const int32_t c = pc[3 * p + a];
        if (c < m) left.push_back(p);
        else if (c > m) right.push_back(p);
        else sep.push_back(p);
      }
      std::vector<int32_t>().swap(pan);
      const int cl = dissect(left);
      const int cr = dissect(right);
      nodes[id].child[0] = cl;
      nodes[id].child[1] = cr;
      nodes[cl].parent = id;
      nodes[cr].parent = id;
      nodes[id].own = std::move(sep);
      return id;
    }
    nodes[id].own = pan;                     // no useful cut: dense leaf
    return id;
  };
  std::vector<int32_t> all(nphi);
  std::iota(all.begin(), all.end(), 0);
  const int root = nphi > 0 ? dissect(all) : -1;
  // ---- postorder (children before parent); elimination position of every panel
  std::vector<int> post;
  post.reserve(nodes.size());
  if (root >= 0) {
    std::vector<std::pair<int, int>> stack{{root, 0}};
    while (!stack.empty()) {
      auto& [nd, state] = stack.back();
      if (state < 2 && nodes[nd].child[state] >= 0) {
        const int c = nodes[nd].child[state];
        state++;
        stack.push_back({c, 0});
      } else if (state < 2) {
        state++;
      } else {
        post.push_back(nd);
        stack.pop_back();
      }
    }
  }
  std::vector<int> fid(nodes.size());          // node -> front index (postorder)
  for (size_t k = 0; k < post.size(); ++k) fid[post[k]] = (int)k;
  std::vector<int64_t> epos(nphi);
  {
    int64_t c = 0;
    for (int nd : post)
      for (int32_t p : nodes[nd].own) epos[p] = c++;
  }
  // ---- adjacency of S (panels sharing a current unknown)
  // ---- boundaries, bottom-up
  const int nfr = (int)post.size();
  std::vector<std::vector<int32_t>> bnd(nfr);
  std::vector<int64_t> mark(nphi, -1);
  for (int f = 0; f < nfr; ++f) {
    const Node& nd = nodes[post[f]];
    int64_t last = -1;
    for (int32_t p : nd.own) last = std::max(last, epos[p]);
    std::vector<int32_t>& B = bnd[f];
    auto consider = [&](int32_t p) {
      if (epos[p] > last && mark[p] != f) {
        mark[p] = f;
        B.push_back(p);
      }
    };
    for (int c = 0; c < 2; ++c)
      if (nd.child[c] >= 0)
        for (int32_t p : bnd[fid[nd.child[c]]]) consider(p);
    for (int32_t j : nd.own)
      for (int32_t k = a_rp[j]; k < a_rp[j + 1]; ++k) {
        const int32_t q = a_col[k];
        for (int32_t kk = t_rp[q]; kk < t_rp[q + 1]; ++kk) consider(t_col[kk]);
      }
    std::sort(B.begin(), B.end(), [&](int32_t a, int32_t b) { return epos[a] < epos[b]; });
  }
  // ---- fronts
  s.fronts.assign(nfr, FrontInfo{});
  std::vector<int32_t> rows, relmap;
  std::vector<AsmEntry> asms;
  std::vector<int32_t> asm_q;
  std::vector<double> asm_c;
  int64_t w_off = 0, u_off = 0;
  std::vector<int32_t> loc(nphi, -1);
  s.flops = 0;
  s.nnz_l = 0;
  s.max_nf = 0;
  for (int f = 0; f < nfr; ++f) {
    const Node& nd = nodes[post[f]];
    FrontInfo& fi = s.fronts[f];
    std::vector<int32_t> own = nd.own;
    std::sort(own.begin(), own.end(), [&](int32_t a, int32_t b) { return epos[a] < epos[b]; });
    fi.ns = (int32_t)own.size();
    fi.nb = (int32_t)bnd[f].size();
    fi.nf = fi.ns + fi.nb;
    fi.parent = nd.parent >= 0 ? fid[nd.parent] : -1;
    fi.child[0] = nd.child[0] >= 0 ? fid[nd.child[0]] : -1;
    fi.child[1] = nd.child[1] >= 0 ? fid[nd.child[1]] : -1;
    fi.w_off = w_off;
    w_off += (int64_t)fi.nf * fi.nf;
    fi.u_off = u_off;
    u_off += fi.nb;
    fi.rows_off = (int64_t)rows.size();
    rows.insert(rows.end(), own.begin(), own.end());
    rows.insert(rows.end(), bnd[f].begin(), bnd[f].end());
    s.max_nf = std::max(s.max_nf, fi.nf);
    s.nnz_l += (int64_t)fi.ns * (fi.ns + 1) / 2 + (int64_t)fi.nb * fi.ns;
    for (int64_t j = 0; j < fi.ns; ++j) {
      const double r = (double)(fi.nf - j);
      s.flops += r * r;   // ~ (nf-j)^2 flops per pivot for the rank-1 update
    }
    // assembly entries: lower triangle of the own columns
    for (int32_t r = 0; r < fi.nf; ++r) loc[rows[fi.rows_off + r]] = r;
    fi.asm_off = (int64_t)asms.size();
    for (int32_t lj = 0; lj < fi.ns; ++lj) {
      const int32_t j = own[lj];
      // gather contributions per row i: sum over shared unknowns q of Ar(i,q) Ar(j,q) D(q)
      std::vector<std::pair<int32_t, std::pair<int32_t, double>>> terms;  // (li, (q, coef))
      for (int32_t k = a_rp[j]; k < a_rp[j + 1]; ++k) {
        const int32_t q = a_col[k];
        const double aj = a_val[k];
        for (int32_t kk = t_rp[q]; kk < t_rp[q + 1]; ++kk) {
          const int32_t i = t_col[kk];
          if (epos[i] < epos[j]) continue;              // upper triangle: assembled as (j, i) earlier
          const int32_t li = loc[i];
          VH_REQUIRE(li >= lj, ERR_UNSUPPORTED, "nested dissection produced an invalid front structure");
          terms.push_back({li, {q, aj * t_val[kk]}});
        }
      }
      std::sort(terms.begin(), terms.end(), [](const auto& a, const auto& b) {
        return a.first != b.first ? a.first < b.first : a.second.first < b.second.first;
      });
      for (size_t t = 0; t < terms.size();) {
        size_t e = t;
        AsmEntry ae;
        ae.li = terms[t].first;
        ae.lj = lj;
        ae.t0 = (int32_t)asm_q.size();
        while (e < terms.size() && terms[e].first == terms[t].first) {
          asm_q.push_back(terms[e].second.first);
          asm_c.push_back(terms[e].second.second);
          ++e;
        }
        ae.t1 = (int32_t)asm_q.size();
        asms.push_back(ae);
        t = e;
      }
    }
    fi.asm_cnt = (int32_t)((int64_t)asms.size() - fi.asm_off);
    for (int32_t r = 0; r < fi.nf; ++r) loc[rows[fi.rows_off + r]] = -1;
  }
  // extend-add maps: child boundary row -> parent local row
  for (int f = 0; f < nfr; ++f) {
    FrontInfo& fi = s.fronts[f];
    fi.relmap_off = (int64_t)relmap.size();
    if (fi.parent < 0) {
      VH_REQUIRE(fi.nb == 0, ERR_UNSUPPORTED, "root front with boundary rows");
      continue;
    }
    const FrontInfo& pf = s.fronts[fi.parent];
    for (int32_t r = 0; r < pf.nf; ++r) loc[rows[pf.rows_off + r]] = r;
    for (int32_t b = 0; b < fi.nb; ++b) {
      const int32_t p = rows[fi.rows_off + fi.ns + b];
      VH_REQUIRE(loc[p] >= 0, ERR_UNSUPPORTED, "child boundary row missing from the parent front");
      relmap.push_back(loc[p]);
    }
    for (int32_t r = 0; r < pf.nf; ++r) loc[rows[pf.rows_off + r]] = -1;
  }
  VH_REQUIRE(asm_q.size() < (size_t)INT32_MAX, ERR_UNSUPPORTED, "assembly lists too large");
  // heights -> levels
  std::vector<int> height(nfr, 0);
  int hmax = 0;
  for (int f = 0; f < nfr; ++f) {
    const FrontInfo& fi = s.fronts[f];
    int h = 0;
    for (int c = 0; c < 2; ++c)
      if (fi.child[c] >= 0) h = std::max(h, height[fi.child[c]] + 1);
    height[f] = h;
    hmax = std::max(hmax, h);
  }
  s.levels.assign(nfr ? hmax + 1 : 0, {});
  for (int f = 0; f < nfr; ++f) s.levels[height[f]].push_back(f);
  s.level_max_ns.assign(s.levels.size(), 0);
  s.level_max_nf.assign(s.levels.size(), 0);
  for (size_t h = 0; h < s.levels.size(); ++h)
    for (int f : s.levels[h]) {
      s.level_max_ns[h] = std::max(s.level_max_ns[h], s.fronts[f].ns);
      s.level_max_nf[h] = std::max(s.level_max_nf[h], s.fronts[f].nf);
    }
  const size_t nh = s.levels.size();
  s.levels_fused.assign(nh, {});
  s.levels_blocked.assign(nh, {});
  s.fused_max_ns.assign(nh, 0);
  s.fused_max_nf.assign(nh, 0);
  s.blocked_max_ns.assign(nh, 0);
  s.blocked_max_nf.assign(nh, 0);
  for (size_t h = 0; h < nh; ++h)
    for (int f : s.levels[h]) {
      const FrontInfo& fi = s.fronts[f];
      const bool fused = fi.nf <= kFusedMaxNf;
      (fused ? s.levels_fused : s.levels_blocked)[h].push_back(f);
      int32_t& mns = (fused ? s.fused_max_ns : s.blocked_max_ns)[h];
      int32_t& mnf = (fused ? s.fused_max_nf : s.blocked_max_nf)[h];
      mns = std::max(mns, fi.ns);
      mnf = std::max(mnf, fi.nf);
    }
  // occupancy classes of the fused fronts: CTAs per SM that the shared memory of a front allows
  // (the kernel holds the packed lower triangle, ns pivots and a 4-pivot panel's column
  // coefficients, 8 bytes each; 228 KB per SM, 1 KB reserved per CTA, at most 16)
  auto ctas_per_sm = [](int nf, int ns) {
    const size_t bytes = ((size_t)nf * (nf + 1) / 2 + (size_t)ns + 4 * (size_t)nf) * 8 + 1024;
    return (int)std::min<size_t>(16, std::max<size_t>(1, (228 * 1024) / bytes));
  };
  s.fused_classes.assign(nh, {});
  for (size_t h = 0; h < nh; ++h) {
    auto& L = s.levels_fused[h];
    std::stable_sort(L.begin(), L.end(), [&](int a, int b) { return s.fronts[a].nf > s.fronts[b].nf; });
    for (size_t i = 0; i < L.size();) {
      const int cls = ctas_per_sm(s.fronts[L[i]].nf, s.fronts[L[i]].ns);
      CholSymbolic::FusedClass fc{(int32_t)i, 0, 0, 0};
      size_t j = i;
      while (j < L.size() && ctas_per_sm(s.fronts[L[j]].nf, s.fronts[L[j]].ns) == cls) {
        fc.max_nf = std::max(fc.max_nf, s.fronts[L[j]].nf);
        fc.max_ns = std::max(fc.max_ns, s.fronts[L[j]].ns);
        ++j;
      }
      fc.count = (int32_t)(j - i);
      s.fused_classes[h].push_back(fc);
      i = j;
    }
  }
  s.nfronts = nfr;
  s.w_total = w_off;
  s.u_total = u_off;
  s.n_asm = (int64_t)asms.size();
  if (getenv("VH_DEBUG_SYMBOLIC")) {
    for (size_t h = 0; h < s.levels.size(); ++h) {
      int64_t sum_ns = 0, sum_nb = 0;
      int max_nb = 0;
      for (int f : s.levels[h]) {
        sum_ns += s.fronts[f].ns;
        sum_nb += s.fronts[f].nb;
        max_nb = std::max(max_nb, s.fronts[f].nb);
      }
      fprintf(stderr, "height %zu: %zu fronts, max ns %d, max nb %d, max nf %d, sum ns %ld, sum nb %ld\n", h,
              s.levels[h].size(), s.level_max_ns[h], max_nb, s.level_max_nf[h], (long)sum_ns, (long)sum_nb);
      for (const auto& fc : s.fused_classes[h])
        fprintf(stderr, "    fused class: %d fronts, max nf %d, max ns %d\n", fc.count, fc.max_nf, fc.max_ns);
    }
  }
  if (!to_device) return;
  // ---- device copies
  upload(s.d_fronts, s.fronts, st);
  upload(s.d_rows, rows, st);
  upload(s.d_relmap, relmap, st);
  upload(s.d_asm, asms, st);
  upload(s.d_asm_q, asm_q, st);
  upload(s.d_asm_c, asm_c, st);
  s.d_levels.assign(s.levels.size(), nullptr);
  for (size_t h = 0; h < s.levels.size(); ++h) upload(s.d_levels[h], s.levels[h], st);
  s.d_levels_fused.assign(nh, nullptr);
  s.d_levels_blocked.assign(nh, nullptr);
  for (size_t h = 0; h < nh; ++h) {
    if (!s.levels_fused[h].empty()) upload(s.d_levels_fused[h], s.levels_fused[h], st);
    if (!s.levels_blocked[h].empty()) upload(s.d_levels_blocked[h], s.levels_blocked[h], st);
  }
  VH_CUDA_TRY(cudaMalloc(&s.d_err, sizeof(int)));
  VH_CUDA_TRY(cudaStreamSynchronize(st));
}

}  // namespace vh
