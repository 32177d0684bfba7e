// Device value cache of a caller-supplied f (CachedFunction, cachedfunction.jl:8-184,
// behind the BatchEvaluator plugin point, batcheval.jl:67-83).
//
// Every task of a solve reads f through the TCI_F_CACHE lookup of
// tci_functions.h: the key of a multi-index is its mixed-radix number split in
// two exact halves, the value sits in an open-addressing table in HBM.  Before a
// group of tasks runs, prefill() makes sure every value those tasks read is in
// the table: a probe kernel checks all (row, column) keys of each task's Pi
// products on the device and compacts the misses; the host turns the misses
// into multi-indices, drops repeats, asks the caller's evaluator for exactly
// those points (in column-major order of first appearance) and an insert
// kernel stores them.  Hits never leave the device.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <vector>

#include "../../include/tci_gb300.h"
#include "fc_slot.h"

namespace tci {

struct Req;
class Engine;

// One Pi product of a task: every row multi-index (sites [0, rl)) joined with
// every column multi-index (sites [rl, rl + cl)); a point list has one empty
// column.  Multi-indices are 0-based bytes.
struct FcProduct {
  const uint8_t* rows;
  int64_t nr;
  int rl;
  const uint8_t* cols;
  int64_t nc;
  int cl;
};
// A distinct missing point: row i joined with column j of product q.
struct FcMiss {
  int32_t q;
  int64_t i, j;
};

// An f computed by the library itself for the points the cache misses (the
// Contraction evaluator of contract(algorithm = :TCI)); it sees the products,
// so it can exploit their row x column structure.
class FEvaluator {
 public:
  virtual ~FEvaluator() = default;
  virtual int values(Engine& e, const std::vector<FcProduct>& prods, const std::vector<FcMiss>& miss,
                     double* out) = 0;
};

struct FCache {
  tci_batch_fn fn = nullptr;   // caller-supplied f, or
  std::shared_ptr<FEvaluator> eval;  // the library's own evaluator
  void* user = nullptr;
  int L = 0;
  int split = 0;               // sites [0, split) form key word 0, [split, L) word 1
  std::vector<int> d;          // local dimensions
  std::vector<int64_t> w;      // mixed-radix weight of each site within its half
  double* params = nullptr;    // the solve's parameter block (TCI_F_CACHE layout)
  tci_fc_entry* table = nullptr;
  uint64_t cap = 0, count = 0;
  int64_t evaluated = 0, calls = 0;
  // scratch: keys and miss lists on the device, their host copies
  void* dscr = nullptr;
  size_t dscr_cap = 0;

  ~FCache();
  // Set up keys for localdims d; params must hold 4 + L doubles.  Values come
  // from fn (with user) or, when fn is null, from eval.
  int init(int L, const int* d, tci_batch_fn fn, void* user, double* params,
           std::shared_ptr<FEvaluator> eval = nullptr);
  // Values of f at every element the tasks in reqs (those with fcache == this)
  // read, stored in the table; writes the table address into params.
  int prefill(Engine& e, const std::vector<Req*>& reqs);
  void release();

 private:
  int grow(uint64_t need, cudaStream_t s);
  int scratch(size_t bytes);
  void write_params();
  void key_of(const uint8_t* v, int len, int site0, int64_t& k0, int64_t& k1) const;
};

// Caller-supplied evaluators by id (tci_f_register).
bool user_fn(int fid, tci_batch_fn* fn, void** user);

// Nonzero while this thread is inside a caller-supplied f: the library may then
// release objects (finalizers) but must not run device work.
int fc_callback_depth();

// Kernels (fcache.cu).
void fc_probe_launch(const tci_fc_entry* tab, uint64_t mask, const int64_t* rk, int64_t nr, const int64_t* ck,
                     int64_t nc, unsigned long long* count, uint64_t* miss, cudaStream_t s);
void fc_insert_launch(tci_fc_entry* tab, uint64_t mask, const tci_fc_entry* in, int64_t n, cudaStream_t s);
void fc_rehash_launch(tci_fc_entry* dst, uint64_t dmask, const tci_fc_entry* src, uint64_t scap, cudaStream_t s);

}  // namespace tci
