// Registered device functions f(v) for batched evaluation over Pi matrices.
//
// In the reference, f is any Julia callable taking a MultiIndex (a vector of
// 1-based local indices, abstracttensortrain.jl:6-7) and filltensor calls it
// once per element of Pi (tensorci2.jl:290-312 -> batcheval.jl:32-61).  Here f
// is a registered device function.  Every registered f is written as
//     f(v) = finish( sum_p term_p(v_p) )
// where the running sums (at most two) are exact in double precision: sums of
// integers below 2^53, or of distinct powers of two spanning at most 53 bits.
// Because they are exact, a row prefix and a column suffix of a multi-index can
// be accumulated separately and added, and the value is bit-identical to the
// one-pass evaluation the CPU oracle performs.  `v` below is the 0-based local
// index (the reference's index minus one).
#pragma once
#include "fc_slot.h"
#include "tci_math.h"

enum {
  TCI_F_LORENTZ = 1,  // coeff / (1 + sum_p v_p^2), v 1-based (test_tensorci2.jl:249)
  TCI_F_SERVED = 2,   // 1/(1 + a sum v^2) + b exp(-g sum (v - c)^2), v and c 1-based
  TCI_F_QTT1D = 3,    // quantics 1-D, x = sum_i b_i 2^-i
  TCI_F_QTT2D = 4,    // quantics 2-D, d = 4: x bit = low bit, y bit = high bit
  TCI_F_DENSE = 5,    // table lookup: f(v) = T[v] (column-major over localdims)
  TCI_F_PRODUCT = 6,  // f(v) = C * prod_n t[n, v_n] from log|t| and sign tables
  TCI_F_CACHE = TCI_FID_CACHE,  // caller-supplied f: values looked up in the solve's device hash table
};

// Parameter layouts (double array `params`):
//   LORENTZ: [coeff]                      (empty => coeff = 1)
//   SERVED : [alpha, beta, gamma, c_1 .. c_L]  (c truncated to integers)
//   QTT1D  : [kind]   kind 0: exp(-x) cos(2000 pi x) + 0.5 exp(-(x-0.3)^2/1e-4)
//                     kind 1: exp(-x)
//                     kind 2: exp(-x) + 1e-4 exp(-2x)
//   QTT2D  : []       exp(-((x-.5)^2 + (y-.5)^2)/0.01) cos(400 pi (x + y))
//   DENSE  : [L, stride_1 .. stride_L, values ...]
//   PRODUCT: [L, D, C, q[L x D], neg[L x D]] (site-major): q = log|t| rounded to a
//            multiple of 2^-40, neg = 1 where t < 0; f = C (-1)^(sum neg) exp(sum q).
//            The rounding makes the sums exact, so f does not depend on how a
//            multi-index is split into row and column parts.
//   CACHE  : [table >> 32, table & 0xffffffff, mask, split, w_1 .. w_L]: the key of v
//            is (k0, k1) = (sum_{p<split} w_p v_p, sum_{p>=split} w_p v_p), mixed-radix
//            weights restarting at 1 at `split`, each half below 2^53 (exact sums);
//            f(v) is the value stored under that key in the open-addressing table
//            of tci_fc_entry slots (linear probing, `mask` + 1 slots).  The host
//            fills the table from the caller's evaluator before any task reads it;
//            a key that is not there reads as NaN.


#define TCI_TWO_THOUSAND_PI 6283.185307179587   /* 2000*pi rounded to double */
#define TCI_FOUR_HUNDRED_PI 1256.6370614359173  /* 400*pi rounded to double  */

TCI_HD void tci_f_term(int fid, const double* params, int site, int v,
                       double* acc0, double* acc1) {
  switch (fid) {
    case TCI_F_LORENTZ: {
      double v1 = (double)(v + 1);
      *acc0 = *acc0 + v1 * v1;
    } break;
    case TCI_F_SERVED: {
      double v1 = (double)(v + 1);
      double dv = v1 - (double)(long long)params[3 + site];  // centres are lattice points
      *acc0 = *acc0 + v1 * v1;
      *acc1 = *acc1 + dv * dv;
    } break;
    case TCI_F_QTT1D: {
      if (v) *acc0 = *acc0 + tci_pow2i(-(site + 1));
    } break;
    case TCI_F_QTT2D: {
      if (v & 1) *acc0 = *acc0 + tci_pow2i(-(site + 1));
      if (v & 2) *acc1 = *acc1 + tci_pow2i(-(site + 1));
    } break;
    case TCI_F_DENSE: {
      *acc0 = *acc0 + (double)v * params[1 + site];
    } break;
    case TCI_F_PRODUCT: {
      const int L = (int)params[0], D = (int)params[1];
      *acc0 = *acc0 + params[3 + site * D + v];
      *acc1 = *acc1 + params[3 + L * D + site * D + v];
    } break;
    case TCI_F_CACHE: {
      const double w = (double)v * params[4 + site];
      if (site < (int)params[3])
        *acc0 = *acc0 + w;
      else
        *acc1 = *acc1 + w;
    } break;
    default: break;
  }
}

// Functions of exact integer sums factor as combine(part0(acc0), part1(acc1)).
// The step kernel tabulates part0/part1 over the integer range a task needs and
// combines per element; the direct path below calls the same three functions,
// so both give identical bits.
//   number of tables: 0 (no factoring), 1 (part0 only) or 2.
TCI_HD int tci_f_tables(int fid) {
  return fid == TCI_F_LORENTZ ? 1 : (fid == TCI_F_SERVED ? 2 : 0);
}
TCI_HD double tci_f_part0(int fid, const double* params, int nparams, double acc0) {
  if (fid == TCI_F_LORENTZ) {
    double coeff = nparams > 0 ? params[0] : 1.0;
    return coeff / (acc0 + 1.0);
  }
  return 1.0 / (1.0 + params[0] * acc0);  // SERVED
}
TCI_HD double tci_f_part1(int fid, const double* params, double acc1) {
  (void)fid;
  return tci_exp(-(params[2] * acc1));  // SERVED
}
// combine(p0, p1) = combine_scaled(p0, scale1(p1)): tables of part1 may hold the
// scaled value, so that combining costs one operation per element.
TCI_HD double tci_f_scale1(int fid, const double* params, double p1) {
  (void)fid;
  return params[1] * p1;  // SERVED
}
TCI_HD double tci_f_combine_scaled(int fid, double p0, double q1) {
  if (fid == TCI_F_LORENTZ) return p0;
  return p0 + q1;  // SERVED
}
TCI_HD double tci_f_combine(int fid, const double* params, double p0, double p1) {
  if (fid == TCI_F_LORENTZ) return p0;
  return tci_f_combine_scaled(fid, p0, tci_f_scale1(fid, params, p1));
}

// Integer form of the per-site terms of the factored functions (exact: the
// double sums of tci_f_term hold the same integers).  Only valid when the
// SERVED centres c are integers.
TCI_HD void tci_f_term_int(int fid, const double* params, int site, int v, long long* acc0, long long* acc1) {
  const long long v1 = v + 1;
  *acc0 += v1 * v1;
  if (fid == TCI_F_SERVED) {
    const long long dv = v1 - (long long)params[3 + site];
    *acc1 += dv * dv;
  }
}

TCI_HD double tci_f_finish(int fid, const double* params, int nparams, double acc0,
                           double acc1) {
  switch (fid) {
    case TCI_F_LORENTZ:
      return tci_f_combine(fid, params, tci_f_part0(fid, params, nparams, acc0), 0.0);
    case TCI_F_SERVED:
      return tci_f_combine(fid, params, tci_f_part0(fid, params, nparams, acc0),
                           tci_f_part1(fid, params, acc1));
    case TCI_F_QTT1D: {
      double x = acc0;
      int kind = nparams > 0 ? (int)params[0] : 0;
      if (kind == 1) return tci_exp(-x);
      if (kind == 2) return tci_exp(-x) + 1e-4 * tci_exp(-(2.0 * x));
      double t1 = tci_exp(-x);
      double t2 = tci_cos(TCI_TWO_THOUSAND_PI * x);
      double dx = x - 0.3;
      double t3 = tci_exp(-(dx * dx) / 1e-4);
      return t1 * t2 + 0.5 * t3;
    }
    case TCI_F_QTT2D: {
      double dx = acc0 - 0.5, dy = acc1 - 0.5;
      double g = tci_exp(-(dx * dx + dy * dy) / 0.01);
      return g * tci_cos(TCI_FOUR_HUNDRED_PI * (acc0 + acc1));
    }
    case TCI_F_DENSE: {
      int L = (int)params[0];
      return params[1 + L + (int64_t)acc0];
    }
    case TCI_F_PRODUCT: {
      const double e = params[2] * tci_exp(acc0);
      return (((long long)acc1) & 1) ? -e : e;
    }
    case TCI_F_CACHE: {
#ifdef __CUDA_ARCH__
      const unsigned long long addr =
          ((unsigned long long)params[0] << 32) | (unsigned long long)params[1];
      const tci_fc_entry* tab = (const tci_fc_entry*)addr;
      const unsigned long long mask = (unsigned long long)params[2];
      const unsigned long long k0 = (unsigned long long)acc0, k1 = (unsigned long long)acc1;
      unsigned long long h = tci_fc_hash(k0, k1) & mask;
      for (unsigned long long q = 0; q <= mask; ++q) {
        const unsigned long long e0 = __ldg(&tab[h].k0);
        if (e0 == k0 && __ldg(&tab[h].k1) == k1) return __ldg(&tab[h].v);
        if (e0 == TCI_FC_EMPTY) break;
        h = (h + 1) & mask;
      }
#endif
      return tci_bits_to_double(0x7ff8000000000000ull);
    }
    default:
      return 0.0;
  }
}
