// C ABI: plan upload / free, entry points, error reporting.
#include <algorithm>
#include <atomic>
#include <climits>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <queue>
#include <string>
#include <vector>

#include "common.cuh"
#include "spmm.cuh"

namespace {

thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

int cuda_fail(cudaError_t e, const char* what) {
  return fail(STILE_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// One device arena per plan: every array is copied into a 256-byte aligned
// slot of a single allocation.
struct Arena {
  std::vector<std::pair<const void*, size_t>> parts;
  std::vector<size_t> offs;
  size_t total = 0;
  size_t add(const void* p, size_t bytes) {
    total = (total + 255) & ~size_t(255);
    offs.push_back(total);
    parts.push_back({p, bytes});
    total += bytes;
    return parts.size() - 1;
  }
};

template <typename T>
bool in_range(const T* a, long n, long lo, long hi) {
  for (long i = 0; i < n; ++i)
    if (a[i] < lo || a[i] >= hi) return false;
  return true;
}

}  // namespace

struct StileSpmmPlan {
  void* arena = nullptr;
  void* tid_buf = nullptr;  // ids in the forward operator's numbering (set_transpose_ids)
  int* err_flag = nullptr;
  stile::SpmmArgs args{};
  int M = 0, K = 0;
  long nnz = 0, ell_n_slots = 0;
  int n_zero_rows = 0;
  const int* zero_rows = nullptr;
  long n_tc_dv = 0;  // tensor-tile nonzeros of the value-gradient list
};

// default of the tensor tiles' value gradients: the row runs (measured
// faster on the GCN graph, 40.7 nonzeros per k-step: the tensor-core kernel
// gathers fewer rows, but each CTA waits for its loads, then its MMAs, per
// 64-feature chunk); stile_spmm_plan_set_dvals_mode(1) and the operator's
// backward tuning select the tensor cores
static int tcdv_auto(const StileSpmmPlan* plan) {
  (void)plan;  // one rule for every plan
  return 0;
}

struct StileSddmmPlan {
  void* arena = nullptr;
  int* err_flag = nullptr;
  stile::SddmmArgs args{};
  int M = 0, K = 0;
  long nnz = 0;
};

extern "C" {

int stile_last_error(char* buf, size_t n) {
  if (!buf || n == 0) return STILE_E_INVALID;
  std::snprintf(buf, n, "%s", g_last_error.c_str());
  return STILE_OK;
}

int64_t stile_launch_count(void) { return g_launches.load(); }

int32_t stile_csr_group_nnz(void) { return stile::kCsrGroupNnz; }

int stile_spmm_plan_upload(const StileSpmmPlanHost* h, StileSpmmPlan** out) {
  if (!h || !out) return fail(STILE_E_INVALID, "null argument");
  *out = nullptr;
  if (h->M < 0 || h->K < 0) return fail(STILE_E_INVALID, "negative shape");
  if (h->tc_n_items < 0 || h->tc_n_ksteps < 0 || h->ell_n_items < 0 || h->ell_n_rows < 0 ||
      h->ell_n_slots < 0 || h->n_zero_rows < 0)
    return fail(STILE_E_INVALID, "negative count");
  const int mode = h->tc_mode;
  if (h->tc_n_items > 0) {
    if (mode != STILE_TC_BF16 && mode != STILE_TC_F16 && mode != STILE_TC_SPLIT_BF16 && mode != STILE_TC_FP8)
      return fail(STILE_E_UNSUPPORTED, "unknown tensor-tile mode");
    if (mode == STILE_TC_FP8) {
      if (!h->tc_row_scale) return fail(STILE_E_INVALID, "fp8 tensor tiles need tc_row_scale");
      for (long i = 0; i < (long)h->tc_n_items * 16; ++i)
        if (!(h->tc_row_scale[i] > 0.f) || !(h->tc_row_scale[i] < 3.0e38f))
          return fail(STILE_E_INVALID, "tc_row_scale must be positive and finite");
    }
    const int want = (mode == STILE_TC_SPLIT_BF16) ? 1024 : 512;
    if (h->tc_kstep_bytes != want) return fail(STILE_E_INVALID, "tc_kstep_bytes does not match mode");
    if (!h->tc_item_kbeg || !h->tc_item_flags || !h->tc_out_rows || !h->tc_cols || !h->tc_vals)
      return fail(STILE_E_INVALID, "missing tensor-tile array");
    // host-side validation: monotone k-step ranges, indices in range
    if (h->tc_item_kbeg[0] != 0 || h->tc_item_kbeg[h->tc_n_items] != h->tc_n_ksteps)
      return fail(STILE_E_INVALID, "tc_item_kbeg does not span the k-steps");
    for (int i = 0; i < h->tc_n_items; ++i)
      if (h->tc_item_kbeg[i + 1] < h->tc_item_kbeg[i])
        return fail(STILE_E_INVALID, "tc_item_kbeg not monotone");
    if (!in_range(h->tc_cols, (long)h->tc_n_ksteps * 16, 0, h->K))
      return fail(STILE_E_INVALID, "tc_cols out of range");
    if (!in_range(h->tc_out_rows, (long)h->tc_n_items * 16, -1, h->M))
      return fail(STILE_E_INVALID, "tc_out_rows out of range");
    if (h->tc_nnz_id && !in_range(h->tc_nnz_id, (long)h->tc_n_ksteps * 256, -1, h->nnz))
      return fail(STILE_E_INVALID, "tc_nnz_id out of range");
  }
  if (h->ell_n_items > 0) {
    if (!h->ell_item_row0 || !h->ell_item_K || !h->ell_item_slot0 || !h->ell_item_flags ||
        !h->ell_out_row || !h->ell_row_len || !h->ell_vals || !h->ell_kidx)
      return fail(STILE_E_INVALID, "missing ELL array");
    if (h->ell_item_row0[0] != 0 || h->ell_item_row0[h->ell_n_items] != h->ell_n_rows)
      return fail(STILE_E_INVALID, "ell_item_row0 does not span the rows");
    for (int i = 0; i < h->ell_n_items; ++i) {
      const long nr = h->ell_item_row0[i + 1] - h->ell_item_row0[i];
      if (nr < 0 || h->ell_item_K[i] <= 0) return fail(STILE_E_INVALID, "bad ELL item shape");
      if (h->ell_item_slot0[i] < 0 || h->ell_item_slot0[i] + nr * h->ell_item_K[i] > h->ell_n_slots)
        return fail(STILE_E_INVALID, "ELL item slots out of range");
      for (long r = 0; r < nr; ++r) {
        const int len = h->ell_row_len[h->ell_item_row0[i] + r];
        if (len < 0 || len > h->ell_item_K[i]) return fail(STILE_E_INVALID, "ell_row_len > K");
      }
    }
    if (!in_range(h->ell_kidx, h->ell_n_slots, 0, h->K))
      return fail(STILE_E_INVALID, "ell_kidx out of range");
    if (!in_range(h->ell_out_row, h->ell_n_rows, -1, h->M))
      return fail(STILE_E_INVALID, "ell_out_row out of range");
    if (h->ell_nnz_id && !in_range(h->ell_nnz_id, h->ell_n_slots, -1, h->nnz))
      return fail(STILE_E_INVALID, "ell_nnz_id out of range");
  }
  if (h->n_zero_rows > 0 && (!h->zero_rows || !in_range(h->zero_rows, h->n_zero_rows, 0, h->M)))
    return fail(STILE_E_INVALID, "zero_rows out of range");

  // tensor-core work chunks: items longer than kChunkSteps k-steps are split
  // into balanced runs that accumulate atomically; the rows of split owned
  // items join the rows zeroed before the kernels.  Chunks are stored longest
  // first so that the persistent kernel's round-robin split is balanced.
  std::vector<int32_t> ck_kbeg, ck_nk, ck_item, ck_flags;
  std::vector<int32_t> zero(h->zero_rows, h->zero_rows + h->n_zero_rows);
  for (int i = 0; i < h->tc_n_items; ++i) {
    const int kb = h->tc_item_kbeg[i], ke = h->tc_item_kbeg[i + 1];
    const int n = ke - kb;
    if (n == 0) {  // no k-steps: an owned item's rows are zero, and no chunk is made
      if (!(h->tc_item_flags[i] & 1))
        for (int r = 0; r < 16; ++r)
          if (h->tc_out_rows[(long)i * 16 + r] >= 0) zero.push_back(h->tc_out_rows[(long)i * 16 + r]);
      continue;
    }
    const int nch = n > stile::kChunkSteps ? (n + stile::kChunkSteps - 1) / stile::kChunkSteps : 1;
    const int per = (n + nch - 1) / nch;
    const bool split = nch > 1;
    const int atomic = (h->tc_item_flags[i] & 1) || split ? 1 : 0;
    for (int c = 0; c < nch; ++c) {
      const int c0 = std::min(kb + c * per, ke), c1 = std::min(kb + (c + 1) * per, ke);
      ck_kbeg.push_back(c0);
      ck_nk.push_back(c1 - c0);
      ck_item.push_back(i);
      ck_flags.push_back(atomic);
    }
    if (split && !(h->tc_item_flags[i] & 1))
      for (int r = 0; r < 16; ++r)
        if (h->tc_out_rows[(long)i * 16 + r] >= 0) zero.push_back(h->tc_out_rows[(long)i * 16 + r]);
  }
  // ELL tiles as a stream of live entries ordered by output row (rows of a
  // community then sit in neighbouring groups, which share B rows in L1),
  // cut into groups of at most `cap` entries at row boundaries.  Row code r stores into C row
  // r; -(r + 1) adds atomically (atomic tiles; pieces of rows longer than a
  // group, whose owned rows are zeroed first).  The capacity is the largest
  // of 64, 32, 16 that still gives every warp the device keeps resident
  // (48 per SM) a group.
  std::vector<int32_t> e_col, e_rc, e_id, e_gptr{0};
  std::vector<float> e_val;
  {
    long live = 0;
    for (int i = 0; i < h->ell_n_items; ++i)
      for (int r = h->ell_item_row0[i]; r < h->ell_item_row0[i + 1]; ++r)
        if (h->ell_out_row[r] >= 0) live += h->ell_row_len[r];
    int dev = 0, sms = 1;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      sms = 1;
    const long warps = (long)sms * 48;
    int cap = stile::kSegNnz;
    while (cap > 16 && live / cap < warps) cap /= 2;
    int fill = 0;
    auto close_group = [&]() {
      if (fill) {
        e_gptr.push_back((int32_t)e_col.size());
        fill = 0;
      }
    };
    auto append = [&](long s0, int k0, int k1, int32_t code) {
      for (int k = k0; k < k1; ++k) {
        e_col.push_back(h->ell_kidx[s0 + k]);
        e_val.push_back(h->ell_vals[s0 + k]);
        e_rc.push_back(code);
        if (h->ell_nnz_id) e_id.push_back(h->ell_nnz_id[s0 + k]);
      }
    };
    struct EllRow {
      int32_t orow, len;
      long s0;
      bool atomic;
    };
    std::vector<EllRow> erows;
    for (int i = 0; i < h->ell_n_items; ++i) {
      const int K = h->ell_item_K[i];
      const bool atomic = (h->ell_item_flags[i] & 1) != 0;
      for (int r = h->ell_item_row0[i]; r < h->ell_item_row0[i + 1]; ++r) {
        const int orow = h->ell_out_row[r], len = h->ell_row_len[r];
        if (orow < 0 || len <= 0) continue;
        erows.push_back({orow, len, h->ell_item_slot0[i] + (long)(r - h->ell_item_row0[i]) * K, atomic});
      }
    }
    std::stable_sort(erows.begin(), erows.end(), [](const EllRow& x, const EllRow& y) { return x.orow < y.orow; });
    for (const EllRow& er : erows) {
      {
        const int orow = er.orow, len = er.len;
        const long s0 = er.s0;
        const bool atomic = er.atomic;
        if (len > cap) {
          close_group();
          if (!atomic) zero.push_back(orow);
          for (int k0 = 0; k0 < len; k0 += cap) {
            append(s0, k0, std::min(len, k0 + cap), -(orow + 1));
            fill = 1;
            close_group();
          }
        } else {
          if (fill + len > cap) close_group();
          append(s0, 0, len, atomic ? -(orow + 1) : orow);
          fill += len;
        }
      }
    }
    close_group();
  }
  const long n_pos = (long)e_col.size();
  if (n_pos > INT32_MAX) return fail(STILE_E_INVALID, "too many ELL entries");

  // Write modes, from the actual coverage of every output row.  The ELL
  // kernel runs first and the tensor-core kernel after it, on one stream.
  //  * A row whose ELL entries form one run (one group) is stored by the
  //    ELL kernel: that initialises the row, so it needs no zeroing.
  //  * A row with several ELL runs (split across groups) is zeroed and all
  //    its ELL runs add atomically.
  //  * A tensor-core chunk adds atomically when one of its rows has an ELL
  //    run or another tensor-core writer; it stores otherwise.  Rows of an
  //    atomic chunk without an ELL run are zeroed.
  //  * Rows nobody writes are zeroed.
  {
    auto row_of_code = [](int32_t c) { return c >= 0 ? c : -c - 1; };
    std::vector<int32_t> ell_runs(h->M, 0), tc_writers(h->M, 0);
    for (size_t g = 0; g + 1 < e_gptr.size(); ++g)
      for (long q = e_gptr[g]; q < e_gptr[g + 1]; ++q) {
        const int32_t r = row_of_code(e_rc[q]);
        if (q == e_gptr[g] || row_of_code(e_rc[q - 1]) != r) ++ell_runs[r];
      }
    for (size_t c = 0; c < ck_item.size(); ++c)
      for (int i = 0; i < 16; ++i) {
        const int32_t r = h->tc_out_rows[(long)ck_item[c] * 16 + i];
        if (r >= 0) ++tc_writers[r];
      }
    for (long q = 0; q < n_pos; ++q) {
      const int32_t r = row_of_code(e_rc[q]);
      e_rc[q] = ell_runs[r] == 1 ? r : -(r + 1);
    }
    std::vector<char> needs_zero(h->M, 0);
    for (size_t c = 0; c < ck_item.size(); ++c) {
      bool atomic = false;
      for (int i = 0; i < 16; ++i) {
        const int32_t r = h->tc_out_rows[(long)ck_item[c] * 16 + i];
        if (r >= 0 && (ell_runs[r] > 0 || tc_writers[r] > 1)) atomic = true;
      }
      ck_flags[c] = atomic ? 1 : 0;
      if (atomic)
        for (int i = 0; i < 16; ++i) {
          const int32_t r = h->tc_out_rows[(long)ck_item[c] * 16 + i];
          if (r >= 0 && ell_runs[r] == 0) needs_zero[r] = 1;
        }
    }
    for (int r = 0; r < h->M; ++r)
      if (ell_runs[r] > 1 || (ell_runs[r] == 0 && tc_writers[r] == 0)) needs_zero[r] = 1;
    // this list replaces the caller's zero rows and the ones noted while
    // splitting: every row that needs zeroing is found above
    zero.clear();
    for (int r = 0; r < h->M; ++r)
      if (needs_zero[r]) zero.push_back(r);
  }

  // packed entries; an entry ends its run when the next one in its group
  // has another row code (or there is none)
  std::vector<int32_t> e_ent((size_t)n_pos * 4);
  for (size_t g = 0; g + 1 < e_gptr.size(); ++g)
    for (long q = e_gptr[g]; q < e_gptr[g + 1]; ++q) {
      int32_t vbits;
      std::memcpy(&vbits, &e_val[q], 4);
      e_ent[q * 4 + 0] = e_col[q];
      e_ent[q * 4 + 1] = vbits;
      const int32_t end = (q + 1 == e_gptr[g + 1] || e_rc[q + 1] != e_rc[q]) ? 1 : 0;
      e_ent[q * 4 + 2] = e_rc[q] * 2 + end;  // row code and run end in one field
      e_ent[q * 4 + 3] = 0;
    }
  std::sort(zero.begin(), zero.end());
  zero.erase(std::unique(zero.begin(), zero.end()), zero.end());
  const long nck = (long)ck_item.size();

  // persistent schedule of the tensor-core kernel: chunks, longest first,
  // each to the least loaded of the kernel's resident CTAs; every CTA's
  // chunks (and their k-steps) are then stored contiguously
  int tc_grid = 0;
  long max_cta_steps = 0;
  std::vector<int32_t> cta_chunk{0};
  std::vector<int32_t> s_cols, s_nnz;
  std::vector<uint8_t> s_vals;
  if (nck > 0) {
    const int resident = stile::tc_persistent_ctas(mode);
    if (resident <= 0) return fail(STILE_E_CUDA, "cannot size the tensor-core grid");
    tc_grid = (int)std::min<long>(resident, nck);
    std::vector<int32_t> by_len(nck);
    for (long c = 0; c < nck; ++c) by_len[c] = (int32_t)c;
    std::stable_sort(by_len.begin(), by_len.end(), [&](int32_t x, int32_t y) { return ck_nk[x] > ck_nk[y]; });
    using Load = std::pair<long, int>;  // (k-steps so far, CTA)
    std::priority_queue<Load, std::vector<Load>, std::greater<Load>> heap;
    for (int b = 0; b < tc_grid; ++b) heap.push({0L, b});
    std::vector<std::vector<int32_t>> owned(tc_grid);
    for (long q = 0; q < nck; ++q) {
      Load l = heap.top();
      heap.pop();
      owned[l.second].push_back(by_len[q]);
      heap.push({l.first + ck_nk[by_len[q]], l.second});
    }
    std::vector<int32_t> order;
    order.reserve(nck);
    for (int b = 0; b < tc_grid; ++b) {
      order.insert(order.end(), owned[b].begin(), owned[b].end());
      cta_chunk.push_back((int32_t)order.size());
    }
    while (!heap.empty()) {
      max_cta_steps = std::max(max_cta_steps, heap.top().first);
      heap.pop();
    }
    // k-steps in schedule order
    const size_t kb = (size_t)h->tc_kstep_bytes;
    s_cols.resize((size_t)h->tc_n_ksteps * 16);
    s_vals.resize((size_t)h->tc_n_ksteps * kb);
    if (h->tc_nnz_id) s_nnz.resize((size_t)h->tc_n_ksteps * 256);
    std::vector<int32_t> kbeg2(nck), nk2(nck), item2(nck), flags2(nck);
    long pos = 0;
    for (long q = 0; q < nck; ++q) {
      const int c = order[q];
      const long src = ck_kbeg[c], n = ck_nk[c];
      std::memcpy(&s_cols[pos * 16], h->tc_cols + src * 16, (size_t)n * 16 * 4);
      std::memcpy(&s_vals[pos * kb], static_cast<const uint8_t*>(h->tc_vals) + src * kb, (size_t)n * kb);
      if (h->tc_nnz_id) std::memcpy(&s_nnz[pos * 256], h->tc_nnz_id + src * 256, (size_t)n * 256 * 4);
      kbeg2[q] = (int32_t)pos;
      nk2[q] = (int32_t)n;
      item2[q] = ck_item[c];
      flags2[q] = ck_flags[c];
      pos += n;
    }
    ck_kbeg.swap(kbeg2);
    ck_nk.swap(nk2);
    ck_item.swap(item2);
    ck_flags.swap(flags2);
    if (pos != h->tc_n_ksteps) return fail(STILE_E_INVALID, "tensor-core chunks do not cover the k-steps");
  }

  // value-gradient entry list from the tiles (needs the nonzero ids)
  std::vector<int32_t> dv_row, dv_col, dv_id;
  long n_tc_dv = 0;  // the list's tensor-core entries come first
  if (h->tc_nnz_id)
    for (int i = 0; i < h->tc_n_items; ++i)
      for (int r = 0; r < 16; ++r) {
        const int orow = h->tc_out_rows[(long)i * 16 + r];
        if (orow < 0) continue;
        for (int ks = h->tc_item_kbeg[i]; ks < h->tc_item_kbeg[i + 1]; ++ks)
          for (int k = 0; k < 16; ++k) {
            const int id = h->tc_nnz_id[(long)ks * 256 + r * 16 + k];
            if (id < 0) continue;
            dv_row.push_back(orow);
            dv_col.push_back(h->tc_cols[(long)ks * 16 + k]);
            dv_id.push_back(id);
          }
      }
  n_tc_dv = (long)dv_id.size();
  if (h->ell_nnz_id)
    for (int i = 0; i < h->ell_n_items; ++i) {
      const int K = h->ell_item_K[i];
      for (int r = h->ell_item_row0[i]; r < h->ell_item_row0[i + 1]; ++r) {
        const int orow = h->ell_out_row[r];
        if (orow < 0) continue;
        const long s0 = h->ell_item_slot0[i] + (long)(r - h->ell_item_row0[i]) * K;
        for (int k = 0; k < h->ell_row_len[r]; ++k) {
          const int id = h->ell_nnz_id[s0 + k];
          if (id < 0) continue;
          dv_row.push_back(orow);
          dv_col.push_back(h->ell_kidx[s0 + k]);
          dv_id.push_back(id);
        }
      }
    }
  const long ndv = (long)dv_id.size();
  // runs of one row, cut at kRunGroup entries and where the tensor-core
  // entries end (the row-run kernel's groups; the tensor-core prefix alone
  // serves the fused backward)
  std::vector<int32_t> dv_gptr{0}, dv_grow;
  int dv_groups_tc = 0;
  for (long t = 0; t < ndv; ++t) {
    const bool cut = t + 1 == ndv || dv_row[t + 1] != dv_row[t] || t + 1 - dv_gptr.back() == stile::kRunGroup ||
                     t + 1 == n_tc_dv;
    if (t + 1 == n_tc_dv) dv_groups_tc = (int)dv_grow.size() + 1;
    if (cut) {
      dv_grow.push_back(dv_row[t]);
      dv_gptr.push_back((int32_t)(t + 1));
    }
  }
  if (ndv > INT32_MAX) return fail(STILE_E_INVALID, "too many nonzeros for the value-gradient list");
  // units of the tensor-tile value-gradient kernel: up to kTcDvUnit k-steps
  // of one chunk (chunks are in schedule order here, their k-steps
  // contiguous)
  std::vector<int32_t> u_ks, u_meta;
  if (h->tc_nnz_id && h->tc_n_items > 0)
    for (long c = 0; c < nck; ++c)
      for (int o = 0; o < ck_nk[c]; o += stile::kTcDvUnit) {
        u_ks.push_back(ck_kbeg[c] + o);
        u_meta.push_back(ck_item[c] * stile::kTcDvUnit + std::min(stile::kTcDvUnit, ck_nk[c] - o) - 1);
      }
  if ((long)h->tc_n_items * stile::kTcDvUnit > INT32_MAX) return fail(STILE_E_INVALID, "too many tensor-tile items");

  Arena ar;
  const long ti = h->tc_n_items, tk = h->tc_n_ksteps;
  size_t i_kbeg = ar.add(h->tc_item_kbeg, ti ? (ti + 1) * 4 : 0);
  size_t i_flags = ar.add(h->tc_item_flags, ti * 4);
  size_t i_orows = ar.add(h->tc_out_rows, ti * 16 * 4);
  // k-step arrays in schedule order (every k-step belongs to exactly one chunk)
  size_t i_cols = ar.add(s_cols.data(), s_cols.size() * 4);
  size_t i_vals = ar.add(s_vals.data(), s_vals.size());
  size_t i_tnid = ar.add(s_nnz.data(), s_nnz.size() * 4);
  size_t i_ctac = ar.add(cta_chunk.data(), cta_chunk.size() * 4);
  size_t i_egptr = ar.add(e_gptr.data(), e_gptr.size() * 4);
  size_t i_eent = ar.add(e_ent.data(), e_ent.size() * 4);
  size_t i_enid = ar.add(e_id.data(), e_id.size() * 4);
  size_t i_zero = ar.add(zero.data(), zero.size() * 4);
  size_t i_ckb = ar.add(ck_kbeg.data(), (size_t)nck * 4);
  size_t i_ckn = ar.add(ck_nk.data(), (size_t)nck * 4);
  size_t i_cki = ar.add(ck_item.data(), (size_t)nck * 4);
  size_t i_ckf = ar.add(ck_flags.data(), (size_t)nck * 4);
  size_t i_dvr = ar.add(dv_row.data(), (size_t)ndv * 4);
  size_t i_dvc = ar.add(dv_col.data(), (size_t)ndv * 4);
  size_t i_dvi = ar.add(dv_id.data(), (size_t)ndv * 4);
  size_t i_dvgp = ar.add(dv_gptr.data(), dv_gptr.size() * 4);
  size_t i_dvgr = ar.add(dv_grow.data(), dv_grow.size() * 4);
  size_t i_uks = ar.add(u_ks.data(), u_ks.size() * 4);
  size_t i_umeta = ar.add(u_meta.data(), u_meta.size() * 4);
  size_t i_err = ar.add(nullptr, 16);
  const bool fp8 = mode == STILE_TC_FP8 && h->tc_n_items > 0;
  size_t i_rsc = ar.add(fp8 ? h->tc_row_scale : nullptr, fp8 ? (size_t)h->tc_n_items * 16 * 4 : 0);
  size_t i_amax = ar.add(nullptr, 16);

  auto* plan = new StileSpmmPlan();
  cudaError_t e = cudaMalloc(&plan->arena, ar.total ? ar.total : 256);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaMalloc(plan)");
  }
  char* base = static_cast<char*>(plan->arena);
  for (size_t i = 0; i < ar.parts.size(); ++i) {
    if (ar.parts[i].first && ar.parts[i].second) {
      e = cudaMemcpy(base + ar.offs[i], ar.parts[i].first, ar.parts[i].second, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        cudaFree(plan->arena);
        delete plan;
        return cuda_fail(e, "cudaMemcpy(plan)");
      }
    }
  }
  plan->err_flag = reinterpret_cast<int*>(base + ar.offs[i_err]);
  e = cudaMemset(plan->err_flag, 0, 16);
  if (e != cudaSuccess) {
    cudaFree(plan->arena);
    delete plan;
    return cuda_fail(e, "cudaMemset(plan)");
  }
  auto P = [&](size_t idx) { return (const void*)(base + ar.offs[idx]); };
  stile::SpmmArgs& a = plan->args;
  a.tc_mode = mode;
  a.K = h->K;
  a.tc_n_items = h->tc_n_items;
  a.tc_n_ksteps = h->tc_n_ksteps;
  a.tc_item_kbeg = (const int*)P(i_kbeg);
  a.tc_item_flags = (const int*)P(i_flags);
  a.tc_out_rows = (const int*)P(i_orows);
  a.tc_cols = (const int*)P(i_cols);
  a.tc_vals = P(i_vals);
  a.tc_nnz_id = h->tc_nnz_id ? (const int*)P(i_tnid) : nullptr;
  a.ell_n_groups = (int)e_gptr.size() - 1;
  a.ell_n_pos = n_pos;
  a.ell_group_ptr = (const int*)P(i_egptr);
  a.ell_entry = (const int4*)P(i_eent);
  a.ell_nnz_id = h->ell_nnz_id ? (const int*)P(i_enid) : nullptr;
  a.err_flag = plan->err_flag;
  a.tc_row_scale = fp8 ? (const float*)P(i_rsc) : nullptr;
  a.tc_xamax = (unsigned*)(base + ar.offs[i_amax]);
  plan->M = h->M;
  plan->K = h->K;
  plan->nnz = h->nnz;
  plan->ell_n_slots = n_pos;
  plan->n_zero_rows = (int)zero.size();
  plan->zero_rows = (const int*)P(i_zero);
  a.tc_n_chunks = h->tc_n_items > 0 ? (int)nck : 0;
  a.dv_n = ndv;
  a.dv_row = (const int*)P(i_dvr);
  a.dv_col = (const int*)P(i_dvc);
  a.dv_id = (const int*)P(i_dvi);
  a.dv_n_groups = (int)dv_grow.size();
  a.dv_n_groups_tc = dv_groups_tc;
  a.dv_gptr = (const int*)P(i_dvgp);
  a.dv_grow = (const int*)P(i_dvgr);
  a.tc_chunk_kbeg = (const int*)P(i_ckb);
  a.tc_chunk_nk = (const int*)P(i_ckn);
  a.tc_grid = tc_grid;
  a.tc_max_cta_steps = (int)max_cta_steps;
  a.tc_cta_chunk = (const int*)P(i_ctac);
  a.tc_chunk_item = (const int*)P(i_cki);
  a.tc_chunk_flags = (const int*)P(i_ckf);
  a.tcdv_n_units = (int)u_ks.size();
  a.tcdv_unit_ks = (const int*)P(i_uks);
  a.tcdv_unit_meta = (const int*)P(i_umeta);
  a.tcdv_id = a.tc_nnz_id;  // the plan's own numbering until set_transpose_ids
  plan->n_tc_dv = n_tc_dv;
  a.tcdv_use = tcdv_auto(plan);  // the row runs until the caller selects the tensor cores
  *out = plan;
  return STILE_OK;
}

int stile_spmm_plan_free(StileSpmmPlan* plan) {
  if (!plan) return STILE_OK;
  if (plan->tid_buf) cudaFree(plan->tid_buf);
  cudaError_t e = cudaFree(plan->arena);
  delete plan;
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree(plan)");
  return STILE_OK;
}

static int check_dense_bf16(long ld, int N, const void* ptr, const char* name) {
  if (!ptr) return fail(STILE_E_INVALID, std::string("null ") + name);
  if (ld < N || (ld % 8) != 0)
    return fail(STILE_E_INVALID, std::string(name) + " (bf16): row stride must be >= N and a multiple of 8");
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0)
    return fail(STILE_E_INVALID, std::string(name) + ": must be 16-byte aligned");
  return STILE_OK;
}

static int check_dense(long ld, int N, const void* ptr, const char* name) {
  if (!ptr) return fail(STILE_E_INVALID, std::string("null ") + name);
  if (ld < N || (ld % 4) != 0)
    return fail(STILE_E_INVALID, std::string(name) + ": row stride must be >= N and a multiple of 4");
  if ((reinterpret_cast<uintptr_t>(ptr) & 15) != 0)
    return fail(STILE_E_INVALID, std::string(name) + ": must be 16-byte aligned");
  return STILE_OK;
}

// value sets of a batched run: ELL records, then tensor-tile images, per head
static size_t values_ell_bytes(const StileSpmmPlan* plan) { return (size_t)plan->ell_n_slots * 16; }
static size_t values_tc_bytes(const StileSpmmPlan* plan) {
  const size_t kb = plan->args.tc_mode == STILE_TC_SPLIT_BF16 ? 1024 : 512;
  return (size_t)plan->args.tc_n_ksteps * kb;
}
static size_t values_tc_offset(const StileSpmmPlan* plan, int heads) {
  return ((size_t)heads * values_ell_bytes(plan) + 255) / 256 * 256;
}

struct Heads {
  int n = 0;                // 0: a single run with the plan's own values
  const void* packed = nullptr;
  long b_stride = 0, c_stride = 0;
};

static int spmm_run(const StileSpmmPlan* plan, const void* B, bool b_bf16, int64_t ldb, float* C, int64_t ldc,
                    int32_t N, void* stream, const Heads& hd = Heads()) {
  stile::begin_call();
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (N <= 0) return fail(STILE_E_INVALID, "N must be positive");
  int rc;
  if (b_bf16) {
    if (!B) return fail(STILE_E_INVALID, "null B");
    if (ldb < N || (ldb % 8) != 0)
      return fail(STILE_E_INVALID, "B (bf16): row stride must be >= N and a multiple of 8");
    if ((reinterpret_cast<uintptr_t>(B) & 15) != 0) return fail(STILE_E_INVALID, "B: must be 16-byte aligned");
    if (plan->args.tc_n_chunks && plan->args.tc_mode != STILE_TC_BF16)
      return fail(STILE_E_UNSUPPORTED, "a bf16 B needs a plan with bf16 tensor tiles");
  } else if ((rc = check_dense(ldb, N, B, "B")) != 0) {
    return rc;
  }
  if ((rc = check_dense(ldc, N, C, "C")) != 0) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  const bool fp8 = plan->args.tc_n_chunks && plan->args.tc_mode == STILE_TC_FP8;
  if (fp8) {
    if (hd.n > 0) return fail(STILE_E_UNSUPPORTED, "fp8 tensor tiles take one value set");
    // B's e4m3 scale: max |B| over the run's operand, by an ordinary launch
    // that every later kernel of the run starts after
    e = cudaMemsetAsync(plan->args.tc_xamax, 0, 4, st);
    if (e == cudaSuccess)
      e = stile::launch_amax(static_cast<const float*>(B), ldb, plan->K, N, plan->args.tc_xamax, st);
    if (e != cudaSuccess) return cuda_fail(e, "amax launch");
    g_launches++;
  }
  // rows without an owned writer start at zero; when they are the majority,
  // one strided memset of C is cheaper than the row list (owned rows are
  // overwritten by their writer anyway)
  bool zero_kernel = false;  // the zero-rows kernel runs right before the ELL kernel
  const int heads = hd.n > 0 ? hd.n : 1;
  if (2L * plan->n_zero_rows >= plan->M) {
    if (heads == 1 || hd.c_stride == (long)plan->M * ldc) {
      e = cudaMemset2DAsync(C, (size_t)ldc * 4, 0, (size_t)N * 4, (size_t)plan->M * heads, st);
    } else {
      e = cudaSuccess;
      for (int h = 0; h < heads && e == cudaSuccess; ++h)
        e = cudaMemset2DAsync(C + (long)h * hd.c_stride, (size_t)ldc * 4, 0, (size_t)N * 4, (size_t)plan->M, st);
    }
    if (e != cudaSuccess) return cuda_fail(e, "zeroing C");
  } else {
    e = stile::launch_zero_rows(plan->zero_rows, plan->n_zero_rows, C, ldc, N, st, heads, hd.c_stride);
    if (e != cudaSuccess) return cuda_fail(e, "zero_rows launch");
    if (plan->n_zero_rows) g_launches++;
    zero_kernel = plan->n_zero_rows > 0;
  }
  stile::SpmmArgs a = plan->args;
  a.B = static_cast<const float*>(B);
  a.b_bf16 = b_bf16 ? 1 : 0;
  a.ldb = ldb;
  a.C = C;
  a.ldc = ldc;
  a.N = N;
  a.n_fchunks = (N + 127) / 128;
  // the ELL kernel initialises the rows it stores; the tensor-core kernel
  // adds to them afterwards (write modes chosen at upload)
  a.ell_lazy_wait = zero_kernel ? 1 : 0;
  if (hd.n > 0) {
    a.heads = hd.n;
    a.b_head_stride = hd.b_stride;
    a.c_head_stride = hd.c_stride;
    const uint8_t* pk = static_cast<const uint8_t*>(hd.packed);
    a.ell_entry = reinterpret_cast<const int4*>(pk);
    a.tc_vals = pk + values_tc_offset(plan, hd.n);
    a.tc_vals_head_stride = (long)values_tc_bytes(plan);
  }
  e = stile::launch_ell(a, st);
  if (e != cudaSuccess) return cuda_fail(e, "ELL SpMM launch");
  if (a.ell_n_groups) g_launches++;
  e = stile::launch_tc(a, st);
  if (e != cudaSuccess) return cuda_fail(e, "tensor-core SpMM launch");
  if (a.tc_n_chunks) g_launches++;
  return STILE_OK;
}

int stile_spmm_run(const StileSpmmPlan* plan, const float* B, int64_t ldb, float* C, int64_t ldc, int32_t N,
                   void* stream) {
  return spmm_run(plan, B, false, ldb, C, ldc, N, stream);
}

int stile_spmm_run_bf16(const StileSpmmPlan* plan, const uint16_t* B, int64_t ldb, float* C, int64_t ldc,
                        int32_t N, void* stream) {
  return spmm_run(plan, B, true, ldb, C, ldc, N, stream);
}

int64_t stile_spmm_values_bytes(const StileSpmmPlan* plan, int32_t heads) {
  if (!plan || heads < 0) return fail(STILE_E_INVALID, "bad arguments");
  return (int64_t)(values_tc_offset(plan, heads) + (size_t)heads * values_tc_bytes(plan));
}

int stile_spmm_values_pack(const StileSpmmPlan* plan, const float* vals, int32_t heads, void* packed, void* stream) {
  stile::begin_call();
  if (!plan || heads < 0) return fail(STILE_E_INVALID, "bad arguments");
  if (plan->args.tc_n_chunks && plan->args.tc_mode == STILE_TC_FP8)
    return fail(STILE_E_UNSUPPORTED, "fp8 tensor tiles take one value set (their scales come with the plan)");
  if (heads == 0) return STILE_OK;
  if (!vals || !packed) return fail(STILE_E_INVALID, "null argument");
  if ((reinterpret_cast<uintptr_t>(packed) & 255) != 0) return fail(STILE_E_INVALID, "packed: must be 256-byte aligned");
  if ((plan->args.tc_n_items && !plan->args.tc_nnz_id) || (plan->args.ell_n_groups && !plan->args.ell_nnz_id))
    return fail(STILE_E_INVALID, "plan was uploaded without nonzero ids");
  uint8_t* pk = static_cast<uint8_t*>(packed);
  cudaError_t e = stile::launch_pack_values(plan->args, vals, plan->nnz, heads, pk, pk + values_tc_offset(plan, heads),
                                            plan->ell_n_slots, (long)values_tc_bytes(plan),
                                            static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "value pack launch");
  g_launches++;
  return STILE_OK;
}

int stile_spmm_run_batched(const StileSpmmPlan* plan, const void* packed, int32_t heads, const float* B, int64_t ldb,
                           int64_t b_head_stride, float* C, int64_t ldc, int64_t c_head_stride, int32_t N,
                           void* stream) {
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (heads <= 0 || !packed) return fail(STILE_E_INVALID, "heads must be positive and packed non-null");
  if (b_head_stride < (int64_t)plan->K * ldb && heads > 1) return fail(STILE_E_INVALID, "B heads overlap");
  if (c_head_stride < (int64_t)plan->M * ldc && heads > 1) return fail(STILE_E_INVALID, "C heads overlap");
  if ((b_head_stride % 4) != 0 || (c_head_stride % 4) != 0)
    return fail(STILE_E_INVALID, "head strides must be multiples of 4 elements");
  Heads hd;
  hd.n = heads;
  hd.packed = packed;
  hd.b_stride = b_head_stride;
  hd.c_stride = c_head_stride;
  return spmm_run(plan, B, false, ldb, C, ldc, N, stream, hd);
}

static int tc_dvals(const stile::SpmmArgs& a, const int* run_ids, const float* X, long ldx, const float* Y, long ldy,
                    float* out, int N, int ell, cudaStream_t st);

static int spmm_dvals(const StileSpmmPlan* plan, const float* dY, int64_t lddy, const void* B, bool b_bf16,
                      int64_t ldb, float* dvals, int32_t N, void* stream) {
  stile::begin_call();
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (N <= 0) return fail(STILE_E_INVALID, "N must be positive");
  if (!dvals) return fail(STILE_E_INVALID, "null dvals");
  if ((plan->args.tc_n_items && !plan->args.tc_nnz_id) ||
      (plan->args.ell_n_groups && !plan->args.ell_nnz_id))
    return fail(STILE_E_INVALID, "plan was uploaded without nonzero ids");
  int rc;
  if ((rc = b_bf16 ? check_dense_bf16(ldb, N, B, "B") : check_dense(ldb, N, B, "B")) != 0) return rc;
  if ((rc = check_dense(lddy, N, dY, "dY")) != 0) return rc;
  stile::SpmmArgs a = plan->args;
  a.B = static_cast<const float*>(B);
  a.b_bf16 = b_bf16 ? 1 : 0;
  a.ldb = ldb;
  a.N = N;
  if (!b_bf16) {
    // this plan's own numbering (set_transpose_ids renumbers for the fused
    // backward only)
    a.tcdv_id = a.tc_nnz_id;
    return tc_dvals(a, a.dv_id, dY, lddy, static_cast<const float*>(B), ldb, dvals, N, 1,
                    static_cast<cudaStream_t>(stream));
  }
  cudaError_t e = stile::launch_dvals(a, dY, lddy, dvals, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "dvals launch");
  g_launches += (a.dv_n > 0);
  return STILE_OK;
}

int stile_spmm_dvals(const StileSpmmPlan* plan, const float* dY, int64_t lddy, const float* B, int64_t ldb,
                     float* dvals, int32_t N, void* stream) {
  return spmm_dvals(plan, dY, lddy, B, false, ldb, dvals, N, stream);
}

int stile_spmm_dvals_bf16(const StileSpmmPlan* plan, const float* dY, int64_t lddy, const uint16_t* B, int64_t ldb,
                          float* dvals, int32_t N, void* stream) {
  return spmm_dvals(plan, dY, lddy, B, true, ldb, dvals, N, stream);
}

int stile_spmm_plan_set_transpose_ids(StileSpmmPlan* plan, const int32_t* perm, int64_t nnz, void* stream) {
  stile::begin_call();
  if (!plan || !perm) return fail(STILE_E_INVALID, "null argument");
  if (nnz != plan->nnz) return fail(STILE_E_INVALID, "perm must have one entry per nonzero of the plan");
  if ((plan->args.tc_n_items && !plan->args.tc_nnz_id) || (plan->args.ell_n_groups && !plan->args.ell_nnz_id))
    return fail(STILE_E_INVALID, "plan was uploaded without nonzero ids");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const long n_ell = plan->args.ell_n_groups ? plan->ell_n_slots : 0, n_dv = plan->args.dv_n;
  const long n_tc = plan->args.tcdv_n_units ? (long)plan->args.tc_n_ksteps * 256 : 0;
  if (!plan->tid_buf) {
    cudaError_t e = cudaMalloc(&plan->tid_buf, (size_t)(n_ell + n_dv + n_tc + 1) * 4);
    if (e != cudaSuccess) {
      plan->tid_buf = nullptr;
      return cuda_fail(e, "cudaMalloc(transpose ids)");
    }
  }
  int* ids = static_cast<int*>(plan->tid_buf);
  // the ELL records carry their id in their fourth word; the run list gets
  // a permuted copy
  cudaError_t e = stile::launch_record_ids(const_cast<int4*>(plan->args.ell_entry), plan->args.ell_nnz_id, n_ell,
                                           perm, st);
  if (e == cudaSuccess) e = stile::launch_permute_ids(plan->args.dv_id, n_dv, perm, ids + n_ell, st);
  if (e == cudaSuccess && n_tc)
    e = stile::launch_permute_ids(plan->args.tc_nnz_id, n_tc, perm, ids + n_ell + n_dv, st);
  if (e != cudaSuccess) return cuda_fail(e, "id permutation launch");
  g_launches += (n_ell > 0) + (n_dv > 0) + (n_tc > 0);
  plan->args.ell_ids_set = 1;
  plan->args.dvp_id = ids + n_ell;
  if (n_tc) plan->args.tcdv_id = ids + n_ell + n_dv;
  return STILE_OK;
}

// Value gradients out[id] = <X[row], Y[col]> over the plan's entry list (ids
// `run_ids` in the run list's order, the tensor-tile ones in a.tcdv_id):
// the tensor-tile nonzeros on the tensor cores when the plan uses them
// (else by the run list's tensor-core prefix), then, with ell != 0, the
// row-tile nonzeros by the rest of the run list.
static int tc_dvals(const stile::SpmmArgs& a, const int* run_ids, const float* X, long ldx, const float* Y, long ldy,
                    float* out, int N, int ell, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (a.tcdv_use) {
    e = stile::launch_tc_dvals(a, X, ldx, Y, ldy, out, N, st);
    if (e != cudaSuccess) return cuda_fail(e, "tensor-tile dvals launch");
    g_launches += (a.tcdv_n_units > 0);
    const int n = a.dv_n_groups - a.dv_n_groups_tc;
    if (ell && n > 0) {
      e = stile::launch_sddmm_runs(n, a.dv_gptr + a.dv_n_groups_tc, a.dv_grow + a.dv_n_groups_tc, a.dv_col, run_ids,
                                   X, false, ldx, Y, false, ldy, out, N, st);
      if (e != cudaSuccess) return cuda_fail(e, "dvals launch");
      g_launches++;
    }
    return STILE_OK;
  }
  const int n = ell ? a.dv_n_groups : a.dv_n_groups_tc;
  e = stile::launch_sddmm_runs(n, a.dv_gptr, a.dv_grow, a.dv_col, run_ids, X, false, ldx, Y, false, ldy, out, N, st);
  if (e != cudaSuccess) return cuda_fail(e, "dvals launch");
  g_launches += (n > 0);
  return STILE_OK;
}

int stile_spmm_plan_set_dvals_mode(StileSpmmPlan* plan, int32_t mode) {
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (mode < 0 || mode > 2) return fail(STILE_E_INVALID, "mode must be 0 (auto), 1 (tensor cores) or 2 (row runs)");
  stile::SpmmArgs& a = plan->args;
  if (mode == 1 && a.tc_n_ksteps > 0 && a.tcdv_n_units == 0)
    return fail(STILE_E_INVALID, "plan was uploaded without nonzero ids");
  a.tcdv_use = mode == 0 ? tcdv_auto(plan) : (mode == 1 && a.tcdv_n_units > 0) ? 1 : 0;
  return STILE_OK;
}

int stile_spmm_backward(const StileSpmmPlan* planT, const float* dC, int64_t lddc, const float* B, int64_t ldb,
                        float* dB, int64_t lddb, float* dvals, int32_t N, void* stream) {
  stile::begin_call();
  if (!planT) return fail(STILE_E_INVALID, "null plan");
  if (N <= 0) return fail(STILE_E_INVALID, "N must be positive");
  if (!dvals) return fail(STILE_E_INVALID, "null dvals");
  if (!planT->args.dvp_id || (planT->args.ell_n_groups && !planT->args.ell_ids_set))
    return fail(STILE_E_INVALID, "call stile_spmm_plan_set_transpose_ids first");
  int rc;
  if ((rc = check_dense(lddc, N, dC, "dC")) != 0) return rc;
  if ((rc = check_dense(ldb, N, B, "B")) != 0) return rc;
  if ((rc = check_dense(lddb, N, dB, "dB")) != 0) return rc;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  stile::SpmmArgs a = planT->args;
  a.B = dC;
  a.b_bf16 = 0;
  a.ldb = lddc;
  a.C = dB;
  a.ldc = lddb;
  a.N = N;
  a.n_fchunks = (N + 127) / 128;
  a.dvx = B;
  a.dvx_ld = ldb;
  a.dv_out = dvals;
  if (N > 128 || !planT->args.ell_n_groups) {
    // wider than one feature pass (or no row tiles): the transposed product,
    // then the gradient of every nonzero from the run list
    if ((rc = spmm_run(planT, dC, false, lddc, dB, lddb, N, stream)) != 0) return rc;
    return tc_dvals(a, a.dvp_id, B, ldb, dC, lddc, dvals, N, 1, st);
  }
  bool zero_kernel = false;
  if (2L * planT->n_zero_rows >= planT->M) {
    e = cudaMemset2DAsync(dB, (size_t)lddb * 4, 0, (size_t)N * 4, (size_t)planT->M, st);
    if (e != cudaSuccess) return cuda_fail(e, "zeroing dB");
  } else {
    e = stile::launch_zero_rows(planT->zero_rows, planT->n_zero_rows, dB, lddb, N, st);
    if (e != cudaSuccess) return cuda_fail(e, "zero_rows launch");
    if (planT->n_zero_rows) g_launches++;
    zero_kernel = planT->n_zero_rows > 0;
  }
  a.ell_lazy_wait = zero_kernel ? 1 : 0;
  e = stile::launch_ell_bwd(a, st);
  if (e != cudaSuccess) return cuda_fail(e, "fused backward ELL launch");
  g_launches++;
  e = stile::launch_tc(a, st);
  if (e != cudaSuccess) return cuda_fail(e, "tensor-core SpMM launch");
  if (a.tc_n_chunks) g_launches++;
  // the tensor-core nonzeros' gradients (rows of A^T hold B's rows,
  // columns dC's): on the tensor cores, or the run list's tensor-core prefix
  if ((rc = tc_dvals(a, a.dvp_id, B, ldb, dC, lddc, dvals, N, 0, st)) != 0) return rc;
  return STILE_OK;
}

int stile_spmm_plan_set_values(StileSpmmPlan* plan, const float* vals, void* stream) {
  stile::begin_call();
  if (!plan || !vals) return fail(STILE_E_INVALID, "null argument");
  if (plan->args.tc_n_chunks && plan->args.tc_mode == STILE_TC_FP8)
    return fail(STILE_E_UNSUPPORTED, "fp8 tensor tiles: new values need a new upload (their row scales change)");
  if ((plan->args.tc_n_items && !plan->args.tc_nnz_id) ||
      (plan->args.ell_n_groups && !plan->args.ell_nnz_id))
    return fail(STILE_E_INVALID, "plan was uploaded without nonzero ids");
  cudaError_t e = stile::launch_repack(plan->args, vals, plan->ell_n_slots,
                                       static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "value re-pack launch");
  g_launches++;
  return STILE_OK;
}

int stile_spmm_plan_error_flag(StileSpmmPlan* plan, void* stream, int32_t* flag) {
  if (!plan || !flag) return fail(STILE_E_INVALID, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int host = 0;
  cudaError_t e = cudaMemcpyAsync(&host, plan->err_flag, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemsetAsync(plan->err_flag, 0, 4, st);
  if (e != cudaSuccess) return cuda_fail(e, "error flag readback");
  *flag = host;
  return STILE_OK;
}

int stile_spmm_plan_set_wait_policy(StileSpmmPlan* plan, int32_t polls, int32_t stall_test) {
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (stall_test && polls <= 0)
    return fail(STILE_E_INVALID, "a stall test needs a poll limit (the default wait lasts seconds)");
  plan->args.poll_limit = polls > 0 ? (uint32_t)polls : 0u;
  plan->args.stall_test = stall_test ? 1 : 0;
  return STILE_OK;
}

int stile_sparse_attention(int32_t n_rows, const int32_t* indptr, const int32_t* indices, const float* Q,
                           const float* K, const float* V, int64_t ldq, int64_t ldk, int64_t ldv,
                           int64_t q_head_stride, int64_t k_head_stride, int64_t v_head_stride, float* out,
                           int64_t ldo, int64_t out_head_stride, int32_t F, int32_t Fv, float scale, int32_t heads,
                           void* stream) {
  stile::begin_call();
  if (n_rows < 0 || heads < 0) return fail(STILE_E_INVALID, "bad shape");
  if (F <= 0 || Fv <= 0 || F > 128 || Fv > 128)
    return fail(STILE_E_UNSUPPORTED, "fused attention takes 1..128 features for Q/K and for V");
  if (n_rows == 0 || heads == 0) return STILE_OK;
  if (!indptr || !indices) return fail(STILE_E_INVALID, "null pattern");
  int rc;
  if ((rc = check_dense(ldq, F, Q, "Q")) != 0) return rc;
  if ((rc = check_dense(ldk, F, K, "K")) != 0) return rc;
  if ((rc = check_dense(ldv, Fv, V, "V")) != 0) return rc;
  if ((rc = check_dense(ldo, Fv, out, "out")) != 0) return rc;
  if (heads > 1 && ((q_head_stride % 4) || (k_head_stride % 4) || (v_head_stride % 4) || (out_head_stride % 4)))
    return fail(STILE_E_INVALID, "head strides must be multiples of 4 elements");
  if (heads > 1 && out_head_stride < (int64_t)n_rows * ldo) return fail(STILE_E_INVALID, "output heads overlap");
  cudaError_t e = stile::launch_sparse_attention(n_rows, indptr, indices, Q, K, V, ldq, ldk, ldv, q_head_stride,
                                                 k_head_stride, v_head_stride, out, ldo, out_head_stride, F, Fv,
                                                 scale, heads, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "sparse attention launch");
  g_launches++;
  return STILE_OK;
}

int stile_sddmm_plan_error_flag(StileSddmmPlan* plan, void* stream, int32_t* flag) {
  if (!plan || !flag) return fail(STILE_E_INVALID, "null argument");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int host = 0;
  cudaError_t e = cudaMemcpyAsync(&host, plan->err_flag, 4, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e == cudaSuccess) e = cudaMemsetAsync(plan->err_flag, 0, 4, st);
  if (e != cudaSuccess) return cuda_fail(e, "error flag readback");
  *flag = host;
  return STILE_OK;
}

int stile_csr_row_softmax(int32_t M, const int32_t* indptr, int64_t nnz, const float* x, float* out, float scale,
                          int32_t batch, void* stream) {
  stile::begin_call();
  if (M < 0 || nnz < 0 || batch < 0) return fail(STILE_E_INVALID, "bad shape");
  if (M > 0 && !indptr) return fail(STILE_E_INVALID, "null indptr");
  if (nnz > 0 && batch > 0 && (!x || !out)) return fail(STILE_E_INVALID, "null values");
  cudaError_t e = stile::launch_csr_row_softmax(M, indptr, (long)nnz, x, out, scale, batch,
                                                static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "row softmax launch");
  g_launches += (M > 0 && batch > 0);
  return STILE_OK;
}

int stile_csr_spmm_run(int32_t M, int64_t nnz, const int32_t* indptr, const int32_t* indices, const float* vals,
                       const int32_t* group_rows, const float* B, int64_t ldb, float* C, int64_t ldc, int32_t N,
                       void* stream) {
  stile::begin_call();
  if (M < 0 || N <= 0) return fail(STILE_E_INVALID, "bad shape");
  if (M == 0) return STILE_OK;
  if (!indptr || !indices || !vals) return fail(STILE_E_INVALID, "null CSR array");
  int rc;
  if ((rc = check_dense(ldb, N, B, "B")) != 0) return rc;
  if ((rc = check_dense(ldc, N, C, "C")) != 0) return rc;
  if (nnz < 0) return fail(STILE_E_INVALID, "negative nnz");
  cudaError_t e = stile::launch_csr_spmm(M, indptr, indices, vals, B, ldb, C, ldc, N, nnz, group_rows,
                                         static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "CSR SpMM launch");
  g_launches++;
  return STILE_OK;
}

int stile_sddmm_plan_upload(const StileSddmmPlanHost* h, StileSddmmPlan** out) {
  if (!h || !out) return fail(STILE_E_INVALID, "null argument");
  *out = nullptr;
  if (h->n_1d < 0 || h->n_blk < 0 || h->n_blk_nnz < 0) return fail(STILE_E_INVALID, "negative count");
  if (h->n_1d > 0) {
    if (!h->mid_idx || !h->j_idx || !h->remap) return fail(STILE_E_INVALID, "missing 1D array");
    if (!in_range(h->mid_idx, h->n_1d, 0, h->M) || !in_range(h->j_idx, h->n_1d, 0, h->K) ||
        !in_range(h->remap, h->n_1d, 0, h->nnz))
      return fail(STILE_E_INVALID, "1D index out of range");
  }
  if (h->n_blk > 0) {
    if (h->bm <= 0 || h->bn <= 0 || h->bm > 16 || h->bn > 16)
      return fail(STILE_E_UNSUPPORTED, "block tiles larger than 16x16");
    if (!h->blk_i || !h->blk_j || !h->blk_indptr || !h->blk_dense_pos || !h->blk_out)
      return fail(STILE_E_INVALID, "missing block array");
    if (h->blk_indptr[0] != 0 || h->blk_indptr[h->n_blk] != h->n_blk_nnz)
      return fail(STILE_E_INVALID, "blk_indptr does not span the entries");
    for (int b = 0; b < h->n_blk; ++b) {
      const int n = h->blk_indptr[b + 1] - h->blk_indptr[b];
      if (n < 0 || n > h->bm * h->bn) return fail(STILE_E_INVALID, "bad blk_indptr");
    }
    if (!in_range(h->blk_i, (long)h->n_blk * h->bm, 0, h->M) ||
        !in_range(h->blk_j, (long)h->n_blk * h->bn, 0, h->K) ||
        !in_range(h->blk_dense_pos, h->n_blk_nnz, 0, h->bm * h->bn) ||
        !in_range(h->blk_out, h->n_blk_nnz, 0, h->nnz))
      return fail(STILE_E_INVALID, "block index out of range");
  }
  // the 1D entries as runs of one row, cut at stile::kRunGroup entries
  std::vector<int32_t> run_ptr{0}, run_row;
  for (long t = 0; t < h->n_1d; ++t) {
    if (t + 1 == h->n_1d || h->mid_idx[t + 1] != h->mid_idx[t] || t + 1 - run_ptr.back() == stile::kRunGroup) {
      run_row.push_back(h->mid_idx[t]);
      run_ptr.push_back((int32_t)(t + 1));
    }
  }
  Arena ar;
  size_t a0 = ar.add(h->mid_idx, (size_t)h->n_1d * 4);
  size_t a1 = ar.add(h->j_idx, (size_t)h->n_1d * 4);
  size_t a2 = ar.add(h->remap, (size_t)h->n_1d * 4);
  size_t a3 = ar.add(h->blk_i, (size_t)h->n_blk * h->bm * 4);
  size_t a4 = ar.add(h->blk_j, (size_t)h->n_blk * h->bn * 4);
  size_t a5 = ar.add(h->blk_indptr, h->n_blk ? (size_t)(h->n_blk + 1) * 4 : 0);
  size_t a6 = ar.add(h->blk_dense_pos, (size_t)h->n_blk_nnz * 4);
  size_t a7 = ar.add(h->blk_out, (size_t)h->n_blk_nnz * 4);
  size_t a8 = ar.add(run_ptr.data(), run_ptr.size() * 4);
  size_t a9 = ar.add(run_row.data(), run_row.size() * 4);
  size_t a10 = ar.add(nullptr, 16);
  auto* plan = new StileSddmmPlan();
  cudaError_t e = cudaMalloc(&plan->arena, ar.total ? ar.total : 256);
  if (e != cudaSuccess) {
    delete plan;
    return cuda_fail(e, "cudaMalloc(plan)");
  }
  char* base = static_cast<char*>(plan->arena);
  for (size_t i = 0; i < ar.parts.size(); ++i) {
    if (ar.parts[i].first && ar.parts[i].second) {
      e = cudaMemcpy(base + ar.offs[i], ar.parts[i].first, ar.parts[i].second, cudaMemcpyHostToDevice);
      if (e != cudaSuccess) {
        cudaFree(plan->arena);
        delete plan;
        return cuda_fail(e, "cudaMemcpy(plan)");
      }
    }
  }
  auto P = [&](size_t idx) { return (const int*)(base + ar.offs[idx]); };
  stile::SddmmArgs& a = plan->args;
  a.n_1d = h->n_1d;
  a.mid_idx = P(a0);
  a.j_idx = P(a1);
  a.remap = P(a2);
  a.n_blk = h->n_blk;
  a.bm = h->bm;
  a.bn = h->bn;
  a.blk_i = P(a3);
  a.blk_j = P(a4);
  a.blk_indptr = P(a5);
  a.blk_dense_pos = P(a6);
  a.blk_out = P(a7);
  a.n_runs = (int)run_row.size();
  a.run_ptr = P(a8);
  a.run_row = P(a9);
  plan->err_flag = (int*)(base + ar.offs[a10]);
  a.err_flag = plan->err_flag;
  e = cudaMemset(plan->err_flag, 0, 16);
  if (e != cudaSuccess) {
    cudaFree(plan->arena);
    delete plan;
    return cuda_fail(e, "cudaMemset(plan)");
  }
  plan->M = h->M;
  plan->K = h->K;
  plan->nnz = h->nnz;
  *out = plan;
  return STILE_OK;
}

int stile_sddmm_plan_free(StileSddmmPlan* plan) {
  if (!plan) return STILE_OK;
  cudaError_t e = cudaFree(plan->arena);
  delete plan;
  if (e != cudaSuccess) return cuda_fail(e, "cudaFree(plan)");
  return STILE_OK;
}

static int sddmm_run(const StileSddmmPlan* plan, const void* X, int64_t ldx, const void* Y, int64_t ldy, bool bf16,
                     float* out, int32_t F, void* stream) {
  stile::begin_call();
  if (!plan) return fail(STILE_E_INVALID, "null plan");
  if (F <= 0) return fail(STILE_E_INVALID, "F must be positive");
  if (plan->nnz == 0) return STILE_OK;  // an empty mask: nothing to compute
  if (!out) return fail(STILE_E_INVALID, "null out");
  int rc;
  if ((rc = bf16 ? check_dense_bf16(ldx, F, X, "X") : check_dense(ldx, F, X, "X")) != 0) return rc;
  if ((rc = bf16 ? check_dense_bf16(ldy, F, Y, "Y") : check_dense(ldy, F, Y, "Y")) != 0) return rc;
  stile::SddmmArgs a = plan->args;
  a.X = static_cast<const float*>(X);
  a.xy_bf16 = bf16 ? 1 : 0;
  a.ldx = ldx;
  a.Y = static_cast<const float*>(Y);
  a.ldy = ldy;
  a.out = out;
  a.F = F;
  cudaError_t e = stile::launch_sddmm(a, static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "SDDMM launch");
  g_launches += (a.n_blk > 0) + (a.n_runs > 0);
  return STILE_OK;
}

int stile_sddmm_run(const StileSddmmPlan* plan, const float* X, int64_t ldx, const float* Y, int64_t ldy, float* out,
                    int32_t F, void* stream) {
  return sddmm_run(plan, X, ldx, Y, ldy, false, out, F, stream);
}

int stile_sddmm_run_bf16(const StileSddmmPlan* plan, const uint16_t* X, int64_t ldx, const uint16_t* Y, int64_t ldy,
                         float* out, int32_t F, void* stream) {
  return sddmm_run(plan, X, ldx, Y, ldy, true, out, F, stream);
}

int stile_debug_umma_probe(const void* a_img, const void* b_img, const uint32_t* desc6,
                           uint32_t idesc, int32_t kind, float* out, int32_t* err, void* stream) {
  if (!a_img || !b_img || !desc6 || !out || !err) return fail(STILE_E_INVALID, "null argument");
  // every address the descriptors can form must stay inside the 8 KB images:
  // at most 16 core-matrix groups along either direction
  for (int i = 0; i < 2; ++i) {
    const uint32_t lbo = desc6[3 * i], sbo = desc6[3 * i + 1], lay = desc6[3 * i + 2];
    if (lbo > 2048 || sbo > 2048 || (lbo & 15) || (sbo & 15))
      return fail(STILE_E_INVALID, "probe strides must be multiples of 16 and <= 2048");
    if (lay != 0 && lay != 2 && lay != 4 && lay != 6) return fail(STILE_E_INVALID, "bad layout type");
  }
  if (kind != 0 && kind != 1 && kind != 2)
    return fail(STILE_E_INVALID, "kind must be 0 (f16), 1 (tf32) or 2 (f8f6f4)");
  cudaError_t e = stile::launch_umma_probe(a_img, b_img, desc6, idesc, (uint32_t)kind, out, err,
                                           static_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "probe launch");
  g_launches++;
  return STILE_OK;
}

}  // extern "C"

namespace stile {
int report_error(int code, const char* msg) { return fail(code, msg); }
void note_launches(int n) { g_launches += n; }
}  // namespace stile
