// Operator application on packed product states (warp per input state).
//
// apply_columns: H|b> for single product states b (upstream finite.applyOp with {b: 1},
//   impurityModel/ed/finite.py:1301-1511), warp per state.  Terms that map a state onto
//   itself ("diagonal" terms, flag bit 0) are listed in term order and then summed by one lane
//   per state, the eight states of a block sharing each FP64 warp instruction (GB300 issues
//   an FP64 add in ~20 cycles per warp instruction whatever the number of active lanes, so a
//   warp-wide sum of one state's hundreds of diagonal terms kept the FP64 pipe busy); the
//   off-diagonal emissions go to a per-warp shared-memory buffer where equal output states
//   are merged in term order.  This reproduces upstream's sequential dict sums bit for bit.
//   Operators whose bucket index fits in shared memory run apply_columns_bucket_kernel
//   instead (same outputs): each state tries only the terms that can act on it.
// apply_vector: raw emissions of an operator on a weighted multi-state psi, in (state, term)
//   order, for a later stable sort + segmented sum.
#include "common.cuh"

namespace edgpu {

struct ColParams {
  const uint64_t* states;
  int64_t n_states;
  const uint64_t* ops;
  const double2* coeff;
  const uint32_t* flags;
  int n_terms;
  Restr restr;
  double weight_min;
  const uint64_t* basis;
  int64_t n_basis;
  int filter;
  const int64_t* offsets;
  int64_t* counts;
  uint64_t* out_states;
  int64_t* out_index;
  double2* out_vals;
  int conj_vals;
  int cap;
  int stage_terms;
  int diag_group;  // bucketed kernel: states per warp whose diagonal sums run one per lane
  int32_t* status;
};

// -x by flipping the sign bit on the integer pipe (an FP64 negation would queue on GB300's
// narrow FP64 pipe, ~64 cycles latency and ~20 cycles of issue per warp instruction)
__device__ __forceinline__ double neg_bits(double x) {
  return __longlong_as_double(__double_as_longlong(x) ^ (long long)0x8000000000000000ull);
}

template <int W>
__device__ __forceinline__ bool filter_pass(const ColParams& p, const uint64_t (&s)[W], int64_t& idx) {
  idx = -1;
  if (p.filter == EDGPU_FILTER_NONE) return true;
  idx = find_state<W>(p.basis, p.n_basis, s);
  return p.filter == EDGPU_FILTER_IN_BASIS ? (idx >= 0) : (idx < 0);
}

template <int W>
__global__ void __launch_bounds__(256) apply_columns_kernel(ColParams p) {
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const int T = p.n_terms;

  const double2* scoeff = p.coeff;
  const uint64_t* sops = p.ops;
  const uint32_t* sflags = p.flags;
  size_t off = 0;
  int cplx = 0;  // some coefficient has a nonzero imaginary part
  if (p.stage_terms) {
    double2* c = reinterpret_cast<double2*>(smem);
    uint64_t* o = reinterpret_cast<uint64_t*>(smem + 16 * (size_t)T);
    uint32_t* f = reinterpret_cast<uint32_t*>(smem + 24 * (size_t)T);
    for (int t = threadIdx.x; t < T; t += blockDim.x) {
      c[t] = p.coeff[t];
      o[t] = p.ops[t];
      f[t] = p.flags[t];
      cplx |= c[t].y != 0.0;
    }
    scoeff = c;
    sops = o;
    sflags = f;
    off = (28 * (size_t)T + 15) & ~(size_t)15;
  } else {
    for (int t = threadIdx.x; t < T; t += blockDim.x) cplx |= p.coeff[t].y != 0.0;
  }
  cplx = __syncthreads_or(cplx);
  const int cap = p.cap;
  const int nwords = (T + 31) >> 5;
  const size_t per_warp = (((size_t)cap * (20 + 8 * W) + 8 * (size_t)nwords) + 15) & ~(size_t)15;
  unsigned char* wbase = smem + off + per_warp * warp;
  double2* wvals = reinterpret_cast<double2*>(wbase);
  uint64_t* wkeys = reinterpret_cast<uint64_t*>(wbase + 16 * (size_t)cap);
  int* wtidx = reinterpret_cast<int*>(wbase + (16 + 8 * W) * (size_t)cap);
  // valid diagonal terms of the warp's state and their odd parities, one bit per term
  uint32_t* wvalid = reinterpret_cast<uint32_t*>(wbase + (20 + 8 * W) * (size_t)cap);
  uint32_t* wodd = wvalid + nwords;
  __shared__ int nd_s[8];
  __shared__ double2 dsum_s[8];
  __shared__ int dfirst_s[8];

  const bool fill = p.offsets != nullptr;
  // block-uniform loop: warp w of the block takes state jb + w
  for (int64_t jb = (int64_t)blockIdx.x * wpb; jb < p.n_states; jb += (int64_t)gridDim.x * wpb) {
    const int64_t j = jb + warp;
    const bool active = j < p.n_states;
    uint64_t s0[W];
#pragma unroll
    for (int q = 0; q < W; ++q) s0[q] = 0;
    if (active) load_state<W>(p.states + j * W, s0);
    int m = 0;
    if (active) {
      for (int base = 0; base < T; base += 32) {
        const int t = base + lane;
        bool valid = false, isdiag = false;
        int par = 0;
        double vre = 0.0, vim = 0.0;
        uint64_t s[W];
#pragma unroll
        for (int q = 0; q < W; ++q) s[q] = s0[q];
        if (t < T) {
          valid = apply_term<W>(s, sops[t], par);
          if (valid) {
            isdiag = (sflags[t] & 1u) != 0;
            if (!isdiag) {
              double2 c = scoeff[t];
              if (par & 1) {
                c.x = neg_bits(c.x);
                c.y = neg_bits(c.y);
              }
              vre = c.x;
              vim = c.y;
            }
          }
        }
        const unsigned bd = __ballot_sync(FULL, valid && isdiag);
        const unsigned bp = __ballot_sync(FULL, valid && isdiag && (par & 1));
        const unsigned bo = __ballot_sync(FULL, valid && !isdiag);
        if (lane == 0) {
          wvalid[base >> 5] = bd;
          wodd[base >> 5] = bp;
        }
        if (bo) {
          const int pos = m + __popc(bo & ((1u << lane) - 1u));
          if (valid && !isdiag && pos < cap) {
#pragma unroll
            for (int q = 0; q < W; ++q) wkeys[(size_t)pos * W + q] = s[q];
            wvals[pos] = make_double2(vre, vim);
            wtidx[pos] = t;
          }
          m += __popc(bo);
        }
      }
    }
    if (lane == 0) nd_s[warp] = active ? 1 : 0;
    __syncwarp();
    __syncthreads();
    // Diagonal sums in term order, lane w of warp 0 for the state of warp w: the sequential
    // FP64 adds of up to eight states share each warp instruction.
    if (warp == 0 && lane < wpb) {
      double re = 0.0, im = 0.0;
      int first = -1;
      if (nd_s[lane]) {
        const uint32_t* V = reinterpret_cast<const uint32_t*>(smem + off + per_warp * lane + (20 + 8 * W) * (size_t)cap);
        const uint32_t* O = V + nwords;
        for (int q = 0; q < nwords; ++q) {
          uint32_t bits = V[q];
          const uint32_t odd = O[q];
          while (bits) {
            const int k = __ffs(bits) - 1;
            bits &= bits - 1;
            const int tq = (q << 5) + k;
            double2 c = scoeff[tq];
            if ((odd >> k) & 1u) {
              c.x = neg_bits(c.x);
              c.y = neg_bits(c.y);
            }
            if (first < 0) {
              re = c.x;
              im = c.y;
              first = tq;
            } else {
              re = __dadd_rn(re, c.x);
              // real operator: every imaginary part is a signed zero, and the sum of signed
              // zeros is -0 only when all of them are -0 (IEEE round to nearest)
              im = cplx ? __dadd_rn(im, c.y)
                        : __longlong_as_double(__double_as_longlong(im) & __double_as_longlong(c.y));
            }
          }
        }
      }
      dsum_s[lane] = make_double2(re, im);
      dfirst_s[lane] = first;
    }
    __syncthreads();
    if (!active) continue;
    const double dre = dsum_s[warp].x, dim = dsum_s[warp].y;
    const int dfirst = dfirst_s[warp];
    if (m > cap) {
      if (lane == 0) {
        atomicExch(p.status, (int32_t)EDGPU_ERR_OVERFLOW);
        if (!fill) p.counts[j] = 0;
      }
      continue;
    }
    // Diagonal entry (output == input state).
    bool dkeep = false;
    int64_t didx = -1;
    if (dfirst >= 0) {
      dkeep = abs2_py(dre, dim) >= p.weight_min && restr_ok<W>(p.restr, s0);
      if (dkeep) dkeep = filter_pass<W>(p, s0, didx);
    }
    int kept = 0;       // kept off-diagonal heads so far (warp uniform)
    int dbefore = 0;    // kept heads with first term index < dfirst
    const int64_t obase = fill ? p.offsets[j] : 0;
    for (int c0 = 0; c0 < m; c0 += 32) {
      const int k = c0 + lane;
      bool keep = false;
      double sre = 0.0, sim = 0.0;
      int64_t idx = -1;
      uint64_t key[W];
      int tk = 0x7fffffff;
      if (k < m) {
#pragma unroll
        for (int q = 0; q < W; ++q) key[q] = wkeys[(size_t)k * W + q];
        bool head = true;
        for (int e = 0; e < k; ++e) {
          if (state_eq<W>(key, wkeys + (size_t)e * W)) {
            head = false;
            break;
          }
        }
        if (head) {
          double2 v = wvals[k];
          sre = v.x;
          sim = v.y;
          for (int e = k + 1; e < m; ++e) {
            if (state_eq<W>(key, wkeys + (size_t)e * W)) {
              double2 u = wvals[e];
              sre = __dadd_rn(sre, u.x);
              sim = __dadd_rn(sim, u.y);
            }
          }
          keep = abs2_py(sre, sim) >= p.weight_min && restr_ok<W>(p.restr, key);
          if (keep) keep = filter_pass<W>(p, key, idx);
          tk = wtidx[k];
        }
      }
      const unsigned bk = __ballot_sync(FULL, keep);
      const unsigned bb = __ballot_sync(FULL, keep && dkeep && tk < dfirst);
      if (fill && keep) {
        const int rank = kept + __popc(bk & ((1u << lane) - 1u)) + ((dkeep && dfirst < tk) ? 1 : 0);
        const int64_t o = obase + rank;
        if (p.out_states) store_state<W>(p.out_states + o * W, key);
        if (p.out_index) p.out_index[o] = idx;
        if (p.out_vals) p.out_vals[o] = make_double2(sre, p.conj_vals ? neg_bits(sim) : sim);
      }
      kept += __popc(bk);
      dbefore += __popc(bb);
    }
    if (!fill) {
      if (lane == 0) p.counts[j] = kept + (dkeep ? 1 : 0);
    } else if (dkeep && lane == 0) {
      const int64_t o = obase + dbefore;
      if (p.out_states) store_state<W>(p.out_states + o * W, s0);
      if (p.out_index) p.out_index[o] = didx;
      if (p.out_vals) p.out_vals[o] = make_double2(dre, p.conj_vals ? neg_bits(dim) : dim);
    }
    __syncwarp();
  }
}

// Bucketed form of apply_columns_kernel for operators with many terms (same outputs, bit for
// bit).  A term can act on a state only if every orbital it creates without annihilating is
// empty there, so the off-diagonal terms are bucketed by one such key orbital (the lowest) and
// a state tries only the buckets of its empty orbitals (plus the terms without a key orbital);
// the diagonal terms form one bucket tried in term order.  Each block builds the buckets of the
// term table in shared memory once (stable: term order within a bucket); warps then run their
// states independently (no block barrier per state):
//   * diagonal sum: lanes test 32 diagonal terms at a time, and the valid signed coefficients
//     are broadcast in term order (shuffles) into one FP64 chain that every lane runs, so the
//     sum is upstream's sequential one;
//   * off-diagonal emissions from the buckets land in the per-warp buffer in bucket order and
//     are put back into term order by a rank sort on the term index before the merge, which is
//     the one of apply_columns_kernel.
constexpr int kBucketWarps = 4;

template <int W>
__device__ __forceinline__ int term_bucket(uint64_t ops, uint32_t flags) {
  constexpr int NKEY = 64 * W;  // key orbitals; NKEY: no key orbital; NKEY + 1: diagonal
  if (flags & 1u) return NKEY + 1;
  int cre[4], ann[4], nc = 0, na = 0;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const uint32_t op = (uint32_t)(ops >> (16 * k)) & 0xFFFFu;
    if (!(op & 0x8000u)) continue;
    const int orb = (int)(op & 0x3FFu);
    if (op & 0x4000u)
      cre[nc++] = orb;
    else
      ann[na++] = orb;
  }
  int key = NKEY;
  for (int a = 0; a < nc; ++a) {
    bool annihilated = false;
    for (int b = 0; b < na; ++b) annihilated |= ann[b] == cre[a];
    if (!annihilated && cre[a] < key) key = cre[a];
  }
  return key;  // orbitals at or beyond NKEY (outside the state) also fall in bucket NKEY
}

// Per-warp shared memory of the bucketed kernel: emissions (value, state, basis index, term
// index, group slot), the hash table (slot, smallest term index, size) and the kept-head
// bitmask over term indices with its prefix counts.
__host__ __device__ inline size_t bucket_warp_bytes(int cap, int W, int T) {
  const size_t nwt = (size_t)((T + 31) >> 5);
  return ((size_t)cap * (16 + 8 * (size_t)W + 8 + 4 + 4 + 12) + nwt * 8 + 32 * 20 + 15) & ~(size_t)15;
}

template <int W>
__global__ void __launch_bounds__(32 * kBucketWarps) apply_columns_bucket_kernel(ColParams p) {
  constexpr int NB = 64 * W + 2;
  constexpr int NOKEY = 64 * W, DIAG = 64 * W + 1;
  extern __shared__ __align__(16) unsigned char smem[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int T = p.n_terms;
  int* bptr = reinterpret_cast<int*>(smem);  // [NB + 1]
  int* cursor = bptr + NB + 1;               // [NB]
  int* blist = cursor + NB;                  // [T]
  const size_t index_bytes = ((size_t)4 * (2 * NB + 1 + T) + 15) & ~(size_t)15;
  // bucket sizes, their scan, then a stable fill by warp 0 (term order within a bucket)
  for (int b = threadIdx.x; b < NB; b += blockDim.x) cursor[b] = 0;
  __syncthreads();
  int cplx = 0;
  for (int t = threadIdx.x; t < T; t += blockDim.x) {
    atomicAdd(&cursor[term_bucket<W>(__ldg(p.ops + t), __ldg(p.flags + t))], 1);
    cplx |= __ldg(&p.coeff[t].y) != 0.0;
  }
  cplx = __syncthreads_or(cplx);
  if (threadIdx.x == 0) {
    int acc = 0;
    for (int b = 0; b < NB; ++b) {
      bptr[b] = acc;
      acc += cursor[b];
      cursor[b] = bptr[b];
    }
    bptr[NB] = acc;
  }
  __syncthreads();
  if (warp == 0) {
    for (int base = 0; base < T; base += 32) {
      const int t = base + lane;
      const int k = t < T ? term_bucket<W>(__ldg(p.ops + t), __ldg(p.flags + t)) : -1;
      const unsigned peers = __match_any_sync(FULL, k);
      if (t < T) blist[cursor[k] + __popc(peers & ((1u << lane) - 1u))] = t;
      __syncwarp();
      if (t < T && (peers & ((1u << lane) - 1u)) == 0) cursor[k] += __popc(peers);
      __syncwarp();
    }
  }
  __syncthreads();

  const int cap = p.cap;
  const int ht = cap;                // hash slots: a power of two, at least m (open addressing)
  const int nwt = (T + 31) >> 5;     // words of the kept-head bitmask over term indices
  const size_t per_warp = bucket_warp_bytes(cap, W, T);
  unsigned char* wbase = smem + index_bytes + per_warp * warp;
  double2* wvals = reinterpret_cast<double2*>(wbase);
  uint64_t* wkeys = reinterpret_cast<uint64_t*>(wbase + 16 * (size_t)cap);
  int64_t* widx = reinterpret_cast<int64_t*>(wbase + (16 + 8 * W) * (size_t)cap);
  int* wtidx = reinterpret_cast<int*>(widx + cap);
  int* wslot = wtidx + cap;
  int* hslot = wslot + cap;
  int* hmin = hslot + ht;
  int* hcnt = hmin + ht;
  unsigned* kbits = reinterpret_cast<unsigned*>(hcnt + ht);
  int* kpre = reinterpret_cast<int*>(kbits + nwt);
  double* gre = reinterpret_cast<double*>(wbase + (((size_t)cap * (16 + 8 * W + 8 + 4 + 4 + 12) + nwt * 8 + 7) & ~(size_t)7));
  double* gim = gre + 32;
  int* gfirst = reinterpret_cast<int*>(gim + 32);
  const bool fill = p.offsets != nullptr;
  const int wpb = blockDim.x >> 5;
  const int64_t nwarps = (int64_t)gridDim.x * wpb;
  const int G = p.diag_group;  // 1: each state's diagonal terms tested 32 at a time
  for (int64_t jg = ((int64_t)blockIdx.x * wpb + warp) * G; jg < p.n_states; jg += nwarps * G) {
  if (G > 1) {
    // the diagonal sums of the group's states, one state per lane, each in term order
    const int64_t jl = jg + lane;
    double re = 0.0, im = 0.0;
    int first = -1;
    if (lane < G && jl < p.n_states) {
      uint64_t s0[W];
      load_state<W>(p.states + jl * W, s0);
      // not needed when the basis filter drops the input state itself
      const bool drop = p.filter == EDGPU_FILTER_NOT_IN_BASIS && find_state<W>(p.basis, p.n_basis, s0) >= 0;
      const int dend = drop ? bptr[DIAG] : bptr[DIAG + 1];
      for (int d = bptr[DIAG]; d < dend; ++d) {
        const int t = blist[d];
        uint64_t s[W];
#pragma unroll
        for (int q = 0; q < W; ++q) s[q] = s0[q];
        int par = 0;
        if (!apply_term<W>(s, __ldg(p.ops + t), par)) continue;
        double2 c = __ldg(&p.coeff[t]);
        if (par & 1) {
          c.x = neg_bits(c.x);
          c.y = neg_bits(c.y);
        }
        if (first < 0) {
          re = c.x;
          im = c.y;
          first = t;
        } else {
          re = __dadd_rn(re, c.x);
          im = cplx ? __dadd_rn(im, c.y) : __longlong_as_double(__double_as_longlong(im) & __double_as_longlong(c.y));
        }
      }
    }
    gre[lane] = re;
    gim[lane] = im;
    gfirst[lane] = first;
    __syncwarp();
  }
  const int gn = (int)((p.n_states - jg) < G ? (p.n_states - jg) : G);
  for (int l = 0; l < gn; ++l) {
    const int64_t j = jg + l;
    uint64_t s0[W];
    load_state<W>(p.states + j * W, s0);
    // diagonal entry: the valid diagonal terms summed in term order (not needed when the
    // basis filter drops the input state itself: its output could not be kept)
    double dre = G > 1 ? gre[l] : 0.0, dim = G > 1 ? gim[l] : 0.0;
    int dfirst = G > 1 ? gfirst[l] : -1;
    const int dend = (G > 1 || (p.filter == EDGPU_FILTER_NOT_IN_BASIS && find_state<W>(p.basis, p.n_basis, s0) >= 0))
                         ? bptr[DIAG]
                         : bptr[DIAG + 1];
    for (int b = bptr[DIAG]; b < dend; b += 32) {
      const int i = b + lane;
      bool valid = false;
      double cx = 0.0, cy = 0.0;
      int t = 0;
      if (i < dend) {
        t = blist[i];
        uint64_t s[W];
#pragma unroll
        for (int q = 0; q < W; ++q) s[q] = s0[q];
        int par = 0;
        valid = apply_term<W>(s, __ldg(p.ops + t), par);
        if (valid) {
          double2 c = __ldg(&p.coeff[t]);
          if (par & 1) {
            c.x = neg_bits(c.x);
            c.y = neg_bits(c.y);
          }
          cx = c.x;
          cy = c.y;
        }
      }
      unsigned vm = __ballot_sync(FULL, valid);
      while (vm) {
        const int src = __ffs(vm) - 1;
        vm &= vm - 1;
        const double x = __shfl_sync(FULL, cx, src), y = __shfl_sync(FULL, cy, src);
        const int ts = __shfl_sync(FULL, t, src);
        if (dfirst < 0) {
          dre = x;
          dim = y;
          dfirst = ts;
        } else {
          dre = __dadd_rn(dre, x);
          // real operator: every imaginary part is a signed zero, and the sum of signed zeros
          // is -0 only when all of them are -0 (IEEE round to nearest)
          dim = cplx ? __dadd_rn(dim, y) : __longlong_as_double(__double_as_longlong(dim) & __double_as_longlong(y));
        }
      }
    }
    // off-diagonal emissions from the buckets of the empty orbitals and the keyless terms
    int m = 0;
    auto run_bucket = [&](int lo, int hi) {
      for (int b = lo; b < hi; b += 32) {
        const int i = b + lane;
        bool valid = false;
        uint64_t s[W];
        double2 c = make_double2(0.0, 0.0);
        int t = 0;
        if (i < hi) {
          t = blist[i];
#pragma unroll
          for (int q = 0; q < W; ++q) s[q] = s0[q];
          int par = 0;
          valid = apply_term<W>(s, __ldg(p.ops + t), par);
          if (valid) {
            c = __ldg(&p.coeff[t]);
            if (par & 1) {
              c.x = neg_bits(c.x);
              c.y = neg_bits(c.y);
            }
          }
        }
        const unsigned bo = __ballot_sync(FULL, valid);
        if (bo) {
          const int pos = m + __popc(bo & ((1u << lane) - 1u));
          if (valid && pos < cap) {
#pragma unroll
            for (int q = 0; q < W; ++q) wkeys[(size_t)pos * W + q] = s[q];
            wvals[pos] = c;
            wtidx[pos] = t;
          }
          m += __popc(bo);
        }
      }
    };
#pragma unroll
    for (int q = 0; q < W; ++q) {
      uint64_t bits = ~s0[q];
      while (bits) {
        const int z = __clzll(bits);  // orbital q * 64 + z (most significant bit first)
        bits &= ~(1ull << (63 - z));
        const int orb = q * 64 + z;
        const int lo = bptr[orb], hi = bptr[orb + 1];
        if (hi > lo) run_bucket(lo, hi);
      }
    }
    run_bucket(bptr[NOKEY], bptr[NOKEY + 1]);
    __syncwarp();  // the emission buffer is complete before other lanes read it
    if (m > cap) {
      if (lane == 0) {
        atomicExch(p.status, (int32_t)EDGPU_ERR_OVERFLOW);
        if (!fill) p.counts[j] = 0;
      }
      __syncwarp();
      continue;
    }
    // Merge equal output states.  A per-warp hash table maps each emission to the group of
    // its output state: the group's head is its member with the smallest term index, its
    // value the members' sum in term order (upstream's sequential dict sums); kept heads set
    // their term index in a bitmask whose prefix counts give each output's rank in term order.
    for (int h = lane; h < ht; h += 32) {
      hslot[h] = -1;
      hmin[h] = 0x7fffffff;
      hcnt[h] = 0;
    }
    for (int q = lane; q < nwt; q += 32) kbits[q] = 0u;
    __syncwarp();
    for (int k = lane; k < m; k += 32) {
      uint64_t key[W];
#pragma unroll
      for (int q = 0; q < W; ++q) key[q] = wkeys[(size_t)k * W + q];
      uint64_t hv = 0x9E3779B97F4A7C15ull;
#pragma unroll
      for (int q = 0; q < W; ++q) {
        hv ^= key[q] + 0x9E3779B97F4A7C15ull + (hv << 6) + (hv >> 2);
        hv *= 0xBF58476D1CE4E5B9ull;
        hv ^= hv >> 31;
      }
      int h = (int)(hv & (uint64_t)(ht - 1));
      for (int probe = 0; probe < ht; ++probe) {  // m <= ht groups: a free or equal slot is found
        const int old = atomicCAS(&hslot[h], -1, k);
        if (old == -1 || state_eq<W>(key, wkeys + (size_t)old * W)) break;
        h = (h + 1) & (ht - 1);
      }
      wslot[k] = h;
      atomicMin(&hmin[h], wtidx[k]);
      atomicAdd(&hcnt[h], 1);
    }
    __syncwarp();
    // heads: value, restriction / weight / basis filters; kept heads mark their term index
    for (int k = lane; k < m; k += 32) {
      const int h = wslot[k], tk = wtidx[k];
      if (tk != hmin[h]) continue;
      uint64_t key[W];
#pragma unroll
      for (int q = 0; q < W; ++q) key[q] = wkeys[(size_t)k * W + q];
      double2 v = wvals[k];
      if (hcnt[h] > 1) {  // the other members in increasing term index
        int cur = tk;
        for (int g = 1; g < hcnt[h]; ++g) {
          int nxt = 0x7fffffff, ne = -1;
          for (int e = 0; e < m; ++e)
            if (wslot[e] == h && wtidx[e] > cur && wtidx[e] < nxt) {
              nxt = wtidx[e];
              ne = e;
            }
          const double2 u = wvals[ne];
          v.x = __dadd_rn(v.x, u.x);
          v.y = __dadd_rn(v.y, u.y);
          cur = nxt;
        }
        wvals[k] = v;  // read back only by this lane
      }
      int64_t idx = -1;
      bool keep = abs2_py(v.x, v.y) >= p.weight_min && restr_ok<W>(p.restr, key);
      if (keep) keep = filter_pass<W>(p, key, idx);
      if (keep) {
        widx[k] = idx;
        atomicOr(&kbits[tk >> 5], 1u << (tk & 31));
      }
    }
    __syncwarp();
    // exclusive prefix counts of kept heads per 32 term indices
    int run = 0;
    for (int q0 = 0; q0 < nwt; q0 += 32) {
      const int q = q0 + lane;
      const int c = q < nwt ? __popc(kbits[q]) : 0;
      int incl = c;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, incl, o);
        if (lane >= o) incl += y;
      }
      if (q < nwt) kpre[q] = run + incl - c;
      run += __shfl_sync(FULL, incl, 31);
    }
    __syncwarp();
    const int kept = run;
    auto kept_below = [&](int t) { return kpre[t >> 5] + __popc(kbits[t >> 5] & ((1u << (t & 31)) - 1u)); };
    // Diagonal entry (output == input state).
    bool dkeep = false;
    int64_t didx = -1;
    if (dfirst >= 0) {
      dkeep = abs2_py(dre, dim) >= p.weight_min && restr_ok<W>(p.restr, s0);
      if (dkeep) dkeep = filter_pass<W>(p, s0, didx);
    }
    if (!fill) {
      if (lane == 0) p.counts[j] = kept + (dkeep ? 1 : 0);
      __syncwarp();
      continue;
    }
    const int64_t obase = p.offsets[j];
    for (int k = lane; k < m; k += 32) {
      const int h = wslot[k], tk = wtidx[k];
      if (tk != hmin[h] || !((kbits[tk >> 5] >> (tk & 31)) & 1u)) continue;
      const int64_t o = obase + kept_below(tk) + ((dkeep && dfirst < tk) ? 1 : 0);
      uint64_t key[W];
#pragma unroll
      for (int q = 0; q < W; ++q) key[q] = wkeys[(size_t)k * W + q];
      const double2 v = wvals[k];
      if (p.out_states) store_state<W>(p.out_states + o * W, key);
      if (p.out_index) p.out_index[o] = widx[k];
      if (p.out_vals) p.out_vals[o] = make_double2(v.x, p.conj_vals ? neg_bits(v.y) : v.y);
    }
    if (dkeep && lane == 0) {
      const int64_t o = obase + (dfirst >= 0 ? kept_below(dfirst) : 0);
      if (p.out_states) store_state<W>(p.out_states + o * W, s0);
      if (p.out_index) p.out_index[o] = didx;
      if (p.out_vals) p.out_vals[o] = make_double2(dre, p.conj_vals ? neg_bits(dim) : dim);
    }
    __syncwarp();
  }
  __syncwarp();  // the group's diagonal sums are read before the next group writes them
  }
}

struct VecParams {
  const uint64_t* states;
  const double2* amps;
  int64_t n_states;
  const uint64_t* ops;
  const double2* coeff;
  int n_terms;
  Restr restr;
  const int64_t* offsets;
  int64_t* counts;
  uint64_t* out_states;
  double2* out_vals;
};

template <int W>
__global__ void __launch_bounds__(256) apply_vector_kernel(VecParams p) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const int wpb = blockDim.x >> 5;
  const bool fill = p.offsets != nullptr;
  for (int64_t j = (int64_t)blockIdx.x * wpb + warp; j < p.n_states; j += (int64_t)gridDim.x * wpb) {
    uint64_t s0[W];
    load_state<W>(p.states + j * W, s0);
    const double2 a = fill ? p.amps[j] : make_double2(0.0, 0.0);
    int64_t run = fill ? p.offsets[j] : 0;
    int cnt = 0;
    for (int base = 0; base < p.n_terms; base += 32) {
      const int t = base + lane;
      uint64_t s[W];
#pragma unroll
      for (int q = 0; q < W; ++q) s[q] = s0[q];
      bool valid = false;
      int par = 0;
      if (t < p.n_terms) {
        valid = apply_term<W>(s, p.ops[t], par);
        if (valid) valid = restr_ok<W>(p.restr, s);
      }
      const unsigned b = __ballot_sync(FULL, valid);
      if (fill && valid) {
        const double2 h = p.coeff[t];
        // CPython complex product (no fused multiply-add), then the sign.
        double re = __dsub_rn(__dmul_rn(a.x, h.x), __dmul_rn(a.y, h.y));
        double im = __dadd_rn(__dmul_rn(a.x, h.y), __dmul_rn(a.y, h.x));
        if (par & 1) {
          re = -re;
          im = -im;
        }
        const int64_t o = run + __popc(b & ((1u << lane) - 1u));
        store_state<W>(p.out_states + o * W, s);
        p.out_vals[o] = make_double2(re, im);
      }
      run += __popc(b);
      cnt += __popc(b);
    }
    if (!fill && lane == 0) p.counts[j] = cnt;
  }
}

}  // namespace edgpu

using namespace edgpu;

extern "C" int edgpu_apply_columns(int n_words, const uint64_t* states, int64_t n_states, const edgpu_terms* terms,
                                   const edgpu_restrictions* restr, double weight_min, const uint64_t* basis,
                                   int64_t n_basis, int filter, const int64_t* offsets, int64_t* counts,
                                   uint64_t* out_states, int64_t* out_index, double* out_vals, int conj_vals,
                                   int scratch_entries, int32_t* status_dev, void* stream) {
  if (!terms || n_states < 0 || !status_dev) return EDGPU_ERR_ARG;
  if (n_states == 0) return EDGPU_OK;
  if (!states || (!offsets && !counts)) return EDGPU_ERR_ARG;
  if (filter != EDGPU_FILTER_NONE && (!basis || n_basis < 0)) return EDGPU_ERR_ARG;
  if (filter != EDGPU_FILTER_NONE && filter != EDGPU_FILTER_IN_BASIS && filter != EDGPU_FILTER_NOT_IN_BASIS)
    return EDGPU_ERR_ARG;
  if (restr && (restr->n < 0 || restr->n > EDGPU_MAX_RESTRICTIONS)) return EDGPU_ERR_ARG;
  if (n_words < 1 || n_words > EDGPU_MAX_WORDS) return EDGPU_ERR_ARG;
  ColParams p{};
  p.states = states;
  p.n_states = n_states;
  p.ops = terms->ops;
  p.coeff = reinterpret_cast<const double2*>(terms->coeff);
  p.flags = terms->flags;
  p.n_terms = terms->n_terms;
  p.restr = make_restr(restr);
  p.weight_min = weight_min;
  p.basis = basis;
  p.n_basis = n_basis;
  p.filter = filter;
  p.offsets = offsets;
  p.counts = counts;
  p.out_states = out_states;
  p.out_index = out_index;
  p.out_vals = reinterpret_cast<double2*>(out_vals);
  p.conj_vals = conj_vals;
  p.cap = scratch_entries > 0 ? scratch_entries : 256;
  p.status = status_dev;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t term_bytes = (28 * (size_t)p.n_terms + 15) & ~(size_t)15;
  const size_t per_warp =
      (((size_t)p.cap * (20 + 8 * (size_t)n_words) + 8 * (size_t)((p.n_terms + 31) / 32)) + 15) & ~(size_t)15;
  // four warps (one state each) per block: ~70 KB of shared memory for a 1200-term operator,
  // so a block also fits beside two CTAs of a Lanczos kernel running on another stream
  const size_t smem_max = 220 * 1024;
  int warps = 4;
  p.stage_terms = 1;
  while (warps > 1 && term_bytes + per_warp * warps > smem_max) warps >>= 1;
  if (term_bytes + per_warp * warps > smem_max) {
    p.stage_terms = 0;
    warps = 8;
    while (warps > 1 && per_warp * warps > smem_max) warps >>= 1;
    if (per_warp * warps > smem_max) return EDGPU_ERR_ARG;
  }
  // the bucketed kernel when its term index and four warps' emission buffers fit
  const int nb_keys = 64 * n_words + 2;
  const size_t index_bytes = ((size_t)4 * (2 * nb_keys + 1 + p.n_terms) + 15) & ~(size_t)15;
  const size_t bucket_warp = bucket_warp_bytes(p.cap, n_words, p.n_terms);
  int bwarps = kBucketWarps;
  while (bwarps > 1 && index_bytes + bucket_warp * bwarps > smem_max) bwarps >>= 1;
  const size_t bucket_smem = index_bytes + bucket_warp * bwarps;
  if (bucket_smem <= smem_max && (p.cap & (p.cap - 1)) == 0) {
    // diagonal sums one state per lane when there are states enough for two groups per warp
    // of a full grid (8 warps resident per SM); below 8 states a group, 32 lanes per state
    const int64_t resident = (int64_t)grid_cap() * 8;
    int64_t g = n_states / (2 * resident);
    p.diag_group = g >= 8 ? (int)(g < 32 ? g : 32) : 1;
    int64_t blocks = (n_states + (int64_t)bwarps * p.diag_group - 1) / ((int64_t)bwarps * p.diag_group);
    const int64_t cap_blocks = (int64_t)grid_cap() * 8;
    if (blocks > cap_blocks) blocks = cap_blocks;
    EDGPU_DISPATCH_W(n_words, {
      cudaFuncSetAttribute(apply_columns_bucket_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bucket_smem);
      apply_columns_bucket_kernel<W><<<(unsigned)blocks, 32 * bwarps, bucket_smem, s>>>(p);
      note_launch();
    });
    return check_launch();
  }
  const size_t smem = (p.stage_terms ? term_bytes : 0) + per_warp * warps;
  const int threads = 32 * warps;
  int64_t blocks = (n_states + warps - 1) / warps;
  const int64_t cap_blocks = (int64_t)grid_cap() * 8;
  if (blocks > cap_blocks) blocks = cap_blocks;
  EDGPU_DISPATCH_W(n_words, {
    cudaFuncSetAttribute(apply_columns_kernel<W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    apply_columns_kernel<W><<<(unsigned)blocks, threads, smem, s>>>(p); note_launch();
  });
  return check_launch();
}

extern "C" int edgpu_apply_vector(int n_words, const uint64_t* states, const double* amps, int64_t n_states,
                                  const edgpu_terms* terms, const edgpu_restrictions* restr, const int64_t* offsets,
                                  int64_t* counts, uint64_t* out_states, double* out_vals, void* stream) {
  if (!terms || n_states < 0) return EDGPU_ERR_ARG;
  if (n_states == 0) return EDGPU_OK;
  if (!states || (!offsets && !counts)) return EDGPU_ERR_ARG;
  if (offsets && (!amps || !out_states || !out_vals)) return EDGPU_ERR_ARG;
  if (restr && (restr->n < 0 || restr->n > EDGPU_MAX_RESTRICTIONS)) return EDGPU_ERR_ARG;
  VecParams p{};
  p.states = states;
  p.amps = reinterpret_cast<const double2*>(amps);
  p.n_states = n_states;
  p.ops = terms->ops;
  p.coeff = reinterpret_cast<const double2*>(terms->coeff);
  p.n_terms = terms->n_terms;
  p.restr = make_restr(restr);
  p.offsets = offsets;
  p.counts = counts;
  p.out_states = out_states;
  p.out_vals = reinterpret_cast<double2*>(out_vals);
  const int threads = 256;
  int64_t blocks = (n_states + 7) / 8;
  const int64_t cap_blocks = (int64_t)grid_cap() * 8;
  if (blocks > cap_blocks) blocks = cap_blocks;
  EDGPU_DISPATCH_W(n_words, { apply_vector_kernel<W><<<(unsigned)blocks, threads, 0, (cudaStream_t)stream>>>(p); note_launch(); });
  return check_launch();
}
