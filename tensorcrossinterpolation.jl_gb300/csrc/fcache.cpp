// Host side of the device value cache of a caller-supplied f (fcache.h) and the
// registry of caller-supplied evaluators (tci_f_register).
#include "fcache.h"

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_set>

#include "engine.h"
#include "fc_slot.h"

namespace tci {
namespace {

std::mutex reg_mu;
std::vector<std::pair<tci_batch_fn, void*>> reg;  // slot k <-> id TCI_F_USER + k; null fn = free

int fc_fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

struct Key {
  uint64_t k0, k1;
  bool operator==(const Key& o) const { return k0 == o.k0 && k1 == o.k1; }
};
struct KeyHash {
  size_t operator()(const Key& k) const { return (size_t)tci_fc_hash(k.k0, k.k1); }
};

struct Prod : FcProduct {
  size_t koff = 0, moff = 0;
  Prod(const uint8_t* r, int64_t nr_, int rl_, const uint8_t* c, int64_t nc_, int cl_)
      : FcProduct{r, nr_, rl_, c, nc_, cl_} {}
};

constexpr uint64_t FC_MIN_CAP = 1ull << 16;

thread_local int cb_depth = 0;

}  // namespace

int fc_callback_depth() { return cb_depth; }

bool user_fn(int fid, tci_batch_fn* fn, void** user) {
  std::lock_guard<std::mutex> lk(reg_mu);
  const int k = fid - TCI_F_USER;
  if (k < 0 || k >= (int)reg.size() || !reg[k].first) return false;
  *fn = reg[k].first;
  *user = reg[k].second;
  return true;
}

FCache::~FCache() { release(); }

void FCache::release() {
  if (table) cudaFree(table);
  table = nullptr;
  cap = count = 0;
  if (dscr) cudaFree(dscr);
  dscr = nullptr;
  dscr_cap = 0;
}

// Mixed-radix weights, v_1 fastest as CachedFunction's coeffs
// (cachedfunction.jl:16-19), split where a half would reach 2^52.
int FCache::init(int L_, const int* d_, tci_batch_fn fn_, void* user_, double* params_,
                 std::shared_ptr<FEvaluator> eval_) {
  L = L_;
  fn = fn_;
  user = user_;
  eval = std::move(eval_);
  params = params_;
  d.assign(d_, d_ + L);
  w.assign(L, 0);
  const uint64_t lim = 1ull << 52;
  uint64_t prod = 1;
  int p = 0;
  while (p < L && prod * (uint64_t)d[p] <= lim) {
    w[p] = (int64_t)prod;
    prod *= (uint64_t)d[p];
    ++p;
  }
  split = p;
  prod = 1;
  for (; p < L; ++p) {
    if (prod * (uint64_t)d[p] > lim)
      return fc_fail(TCI_ERR_ARG, "caller-supplied f: prod(localdims) must stay below 2^104 (cache keys)");
    w[p] = (int64_t)prod;
    prod *= (uint64_t)d[p];
  }
  write_params();
  return 0;
}

void FCache::write_params() {
  const uint64_t a = (uint64_t)(uintptr_t)table;
  params[0] = (double)(a >> 32);
  params[1] = (double)(a & 0xffffffffull);
  params[2] = (double)(cap ? cap - 1 : 0);
  params[3] = (double)split;
  for (int p = 0; p < L; ++p) params[4 + p] = (double)w[p];
}

void FCache::key_of(const uint8_t* v, int len, int site0, int64_t& k0, int64_t& k1) const {
  k0 = k1 = 0;
  for (int q = 0; q < len; ++q) {
    const int p = site0 + q;
    (p < split ? k0 : k1) += w[p] * (int64_t)v[q];
  }
}

int FCache::scratch(size_t bytes) {
  if (bytes <= dscr_cap) return 0;
  if (dscr) cudaFree(dscr);
  dscr = nullptr;
  dscr_cap = 0;
  const size_t want = std::max(bytes, (size_t)1 << 20);
  if (cudaMalloc(&dscr, want) != cudaSuccess) {
    cudaGetLastError();
    return fc_fail(TCI_ERR_OOM, "device memory for the f cache's scratch");
  }
  dscr_cap = want;
  return 0;
}

int FCache::grow(uint64_t need, cudaStream_t s) {
  if (table && need * 2 <= cap) return 0;
  uint64_t nc = std::max(cap, FC_MIN_CAP);
  while (nc < need * 2) nc <<= 1;
  tci_fc_entry* nt = nullptr;
  if (cudaMalloc(&nt, nc * sizeof(tci_fc_entry)) != cudaSuccess) {
    cudaGetLastError();
    return fc_fail(TCI_ERR_OOM, "device memory for the f cache");
  }
  cudaMemsetAsync(nt, 0xff, nc * sizeof(tci_fc_entry), s);
  if (table) fc_rehash_launch(nt, nc - 1, table, cap, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) {
    cudaFree(nt);
    return fc_fail(TCI_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  }
  if (table) cudaFree(table);
  table = nt;
  cap = nc;
  write_params();
  return 0;
}

int FCache::prefill(Engine& e, const std::vector<Req*>& reqs) {
  cudaStream_t s = e.stream();
  std::vector<Prod> prods;
  std::vector<std::vector<uint8_t>> owned;  // line-scan points of SEARCH tasks
  for (Req* r : reqs) {
    if (r->fcache != this) continue;
    const tci_task& t = r->t;
    switch (t.kind) {
      case TCI_TASK_RRLU:
        if (!r->ain_host) prods.push_back({r->rows, t.m, t.nl, r->cols, t.n, t.nr});
        break;
      case TCI_TASK_CORE:
        prods.push_back({r->rows, t.m, t.nl, r->cols, t.n, t.nr});
        break;
      case TCI_TASK_SITE:
        prods.push_back({r->rows, t.m, t.nl, r->cols, t.r, t.nr});
        prods.push_back({r->prows, t.r, t.nl, r->cols, t.r, t.nr});
        break;
      case TCI_TASK_EVAL:
        prods.push_back({r->rows, t.m, L, nullptr, 1, 0});
        break;
      case TCI_TASK_SEARCH: {  // the start with one site changed, in (site, value) order
        std::vector<uint8_t> pts;
        for (int p = 0; p < L; ++p)
          for (int v = 0; v < d[p]; ++v) {
            pts.insert(pts.end(), r->rows, r->rows + L);
            pts[pts.size() - L + p] = (uint8_t)v;
          }
        owned.push_back(std::move(pts));
        prods.push_back({owned.back().data(), (int64_t)(owned.back().size() / L), L, nullptr, 1, 0});
      } break;
      default:
        break;
    }
  }
  if (!table) {
    int rc = grow(0, s);
    if (rc) return rc;
  }
  size_t nk = 0, nm = 0;
  for (Prod& p : prods) {
    if (p.nr <= 0 || p.nc <= 0) p.nr = p.nc = 0;
    p.koff = nk;
    nk += 2 * (size_t)(p.nr + p.nc);
    p.moff = nm;
    nm += (size_t)p.nr * (size_t)p.nc;
  }
  if (nm == 0) return 0;
  std::vector<int64_t> hk(nk);
  for (const Prod& p : prods) {
    int64_t* rk = hk.data() + p.koff;
    int64_t* ck = rk + 2 * p.nr;
    for (int64_t i = 0; i < p.nr; ++i) key_of(p.rows + (size_t)i * p.rl, p.rl, 0, rk[2 * i], rk[2 * i + 1]);
    for (int64_t j = 0; j < p.nc; ++j) {
      if (p.cl)
        key_of(p.cols + (size_t)j * p.cl, p.cl, p.rl, ck[2 * j], ck[2 * j + 1]);
      else
        ck[2 * j] = ck[2 * j + 1] = 0;
    }
  }
  const size_t kbytes = (nk * 8 + 255) / 256 * 256;
  const size_t cbytes = (prods.size() * 8 + 255) / 256 * 256;
  int rc = scratch(kbytes + cbytes + nm * 8);
  if (rc) return rc;
  int64_t* dk = (int64_t*)dscr;
  unsigned long long* dcnt = (unsigned long long*)((char*)dscr + kbytes);
  uint64_t* dmiss = (uint64_t*)((char*)dscr + kbytes + cbytes);
  cudaMemcpyAsync(dk, hk.data(), nk * 8, cudaMemcpyHostToDevice, s);
  cudaMemsetAsync(dcnt, 0, prods.size() * 8, s);
  for (size_t q = 0; q < prods.size(); ++q) {
    const Prod& p = prods[q];
    fc_probe_launch(table, cap - 1, dk + p.koff, p.nr, dk + p.koff + 2 * p.nr, p.nc, dcnt + q, dmiss + p.moff, s);
  }
  std::vector<unsigned long long> cnt(prods.size());
  cudaMemcpyAsync(cnt.data(), dcnt, prods.size() * 8, cudaMemcpyDeviceToHost, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return fc_fail(TCI_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  size_t total = 0;
  for (auto c : cnt) total += (size_t)c;
  if (total == 0) return 0;
  std::vector<uint64_t> miss(total);
  {
    size_t at = 0;
    for (size_t q = 0; q < prods.size(); ++q) {
      if (cnt[q]) cudaMemcpyAsync(miss.data() + at, dmiss + prods[q].moff, cnt[q] * 8, cudaMemcpyDeviceToHost, s);
      at += cnt[q];
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
      return fc_fail(TCI_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  }
  // distinct missing points, column-major within each product (the fill order of
  // filltensor), products in task order
  std::unordered_set<Key, KeyHash> seen;
  seen.reserve(total * 2);
  std::vector<tci_fc_entry> ent;
  std::vector<FcMiss> um;
  size_t at = 0;
  for (size_t q = 0; q < prods.size(); ++q) {
    const Prod& p = prods[q];
    uint64_t* m = miss.data() + at;
    std::sort(m, m + cnt[q]);
    const int64_t* rk = hk.data() + p.koff;
    const int64_t* ck = rk + 2 * p.nr;
    for (size_t x = 0; x < cnt[q]; ++x) {
      const int64_t i = (int64_t)(m[x] & 0xffffffffull), j = (int64_t)(m[x] >> 32);
      const Key k{(uint64_t)(rk[2 * i] + ck[2 * j]), (uint64_t)(rk[2 * i + 1] + ck[2 * j + 1])};
      if (!seen.insert(k).second) continue;
      ent.push_back(tci_fc_entry{k.k0, k.k1, 0.0, 0});
      um.push_back(FcMiss{(int32_t)q, i, j});
    }
    at += cnt[q];
  }
  const int64_t u = (int64_t)ent.size();
  std::vector<double> vals((size_t)u);
  if (fn) {
    std::vector<int64_t> pts;
    pts.reserve((size_t)u * L);
    for (const FcMiss& x : um) {
      const Prod& p = prods[(size_t)x.q];
      const uint8_t* a = p.rows + (size_t)x.i * p.rl;
      for (int c = 0; c < p.rl; ++c) pts.push_back((int64_t)a[c] + 1);
      const uint8_t* b = p.cols ? p.cols + (size_t)x.j * p.cl : nullptr;
      for (int c = 0; c < p.cl; ++c) pts.push_back((int64_t)b[c] + 1);
    }
    ++cb_depth;
    const int frc = fn(user, L, u, pts.data(), vals.data());
    --cb_depth;
    if (frc) return fc_fail(TCI_ERR_GENERIC, "caller-supplied f failed (code " + std::to_string(frc) + ")");
  } else {
    std::vector<FcProduct> views(prods.begin(), prods.end());
    ++cb_depth;  // the evaluator may call back into a caller-supplied value map
    const int erc = eval->values(e, views, um, vals.data());
    --cb_depth;
    if (erc) return erc;
  }
  ++calls;
  evaluated += u;
  for (int64_t k = 0; k < u; ++k) ent[(size_t)k].v = vals[(size_t)k];
  rc = grow(count + (uint64_t)u, s);
  if (rc) return rc;
  rc = scratch((size_t)u * sizeof(tci_fc_entry));
  if (rc) return rc;
  cudaMemcpyAsync(dscr, ent.data(), (size_t)u * sizeof(tci_fc_entry), cudaMemcpyHostToDevice, s);
  fc_insert_launch(table, cap - 1, (const tci_fc_entry*)dscr, u, s);
  if (cudaStreamSynchronize(s) != cudaSuccess) return fc_fail(TCI_ERR_CUDA, cudaGetErrorString(cudaGetLastError()));
  count += (uint64_t)u;
  return 0;
}

}  // namespace tci

using namespace tci;

extern "C" int tci_f_register(tci_batch_fn fn, void* user, int32_t* fid) {
  if (!fn || !fid) return fc_fail(TCI_ERR_ARG, "tci_f_register: null evaluator");
  std::lock_guard<std::mutex> lk(reg_mu);
  size_t k = 0;
  while (k < reg.size() && reg[k].first) ++k;
  if (k == reg.size()) reg.emplace_back(nullptr, nullptr);
  reg[k] = {fn, user};
  *fid = (int32_t)(TCI_F_USER + k);
  return 0;
}

extern "C" int tci_f_unregister(int32_t fid) {
  std::lock_guard<std::mutex> lk(reg_mu);
  const int k = fid - TCI_F_USER;
  if (k < 0 || k >= (int)reg.size() || !reg[k].first) return fc_fail(TCI_ERR_ARG, "unknown caller-supplied f");
  reg[k] = {nullptr, nullptr};
  return 0;
}
