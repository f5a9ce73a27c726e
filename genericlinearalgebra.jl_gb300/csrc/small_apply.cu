// Replay of the logged Givens rotations on the rows of Q, then the stable
// ascending sort of the eigenpairs. One CTA per matrix, Q staged in shared
// memory, one thread per row of Q.
//
// Replaces, per matrix:
//   _updateVectors! (GenericLinearAlgebra.jl src/eigenSelfAdjoint.jl:121-128)
//     as called from singleShiftQL! (:404), singleShiftQR! (:439, with -s)
//     and eig2x2! (:158);
//   LinearAlgebra.sorteig! with eigsortby (:592-599): stable ascending.
//
// A sweep touches columns (i, i+1) for consecutive i, so each row keeps the
// column shared by two neighbouring rotations in a register ("carry"): one
// shared-memory load, one store and four FP arithmetic instructions per row
// per rotation. Rotations are staged through shared memory in chunks.
#include "gla_launch.h"
#include "gla_small.cuh"

namespace gla {

constexpr int kRotChunk = 512;

size_t apply_smem_bytes(int n, int elem) {
  // S[n*(n+1)] | rotation chunk (2*kRotChunk) | keys (u64, n) | rank (int, n) | headers (3n+4)
  return (size_t)elem * ((size_t)n * (n + 1) + 2 * kRotChunk) + 8 * (size_t)n + 4 * (size_t)n +
         4 * (3 * (size_t)n + 4) + 16;
}

// V: Q in (from k_tridiag or a previous pass) and the rotated, sorted
// eigenvectors out (same arena, column-major, ld = n). dg: final d (unsorted).
// wout/Vout_final: sorted outputs written only once the chase is done; for
// the reduced-precision run they are the FP32 workspace copies.
// scale_exp: eigenvalues are multiplied by 2^scale_exp on output (may be null).
// ROWS2 (eigen2!): V holds only rows 1 and n of the eigenvector matrix,
// 2 x n column-major at twice the matrix's w offset; the same replay and sort
// on those two rows.
template <class T, bool ROWS2>
__global__ void __launch_bounds__(128) k_apply(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                               T* __restrict__ V, const T* __restrict__ dg_all,
                                               T* __restrict__ wout, ChaseState* __restrict__ cst,
                                               const T* __restrict__ rot, const unsigned* __restrict__ hdr,
                                               const int* __restrict__ info, const int* __restrict__ scale_exp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  ChaseState st = cst[mid];
  if (st.applied) return;
  const bool done = st.status == kChaseDone;
  if (!done && st.nhdr == 0) return;  // nothing logged for this matrix in this pass
  const int n = dsc.n;
  const int nr = ROWS2 ? 2 : n;   // rows held
  const int ld = ROWS2 ? 2 : n + 1;
  const int tid = threadIdx.x, NT = blockDim.x;
  T* S = reinterpret_cast<T*>(smem_raw);
  T* buf = S + (size_t)n * ld;
  unsigned long long* keys = reinterpret_cast<unsigned long long*>(buf + 2 * kRotChunk);
  int* rank = reinterpret_cast<int*>(keys + n);
  T* Vg = V + (ROWS2 ? 2 * dsc.w_off : dsc.a_off);  // column-major, leading dimension nr

  if (info[mid] == -1) {  // non-finite input: NaN outputs
    const T nanv = (T)NAN;
    for (int idx = tid; idx < nr * n; idx += NT) Vg[idx] = nanv;
    for (int i = tid; i < n; i += NT) wout[dsc.w_off + i] = nanv;
    if (tid == 0) cst[mid].applied = 1;
    return;
  }

  for (int j = 0; j < n; j++)
    for (int i = tid; i < nr; i += NT) S[(size_t)j * ld + i] = Vg[(size_t)j * nr + i];
  __syncthreads();

  // ---- replay this pass's rotations: whole sweeps per staged chunk
  const T* myrot = rot + 2 * dsc.rot_off;
  unsigned* hs = reinterpret_cast<unsigned*>(rank + n);
  const int nhdr = st.nhdr;
  for (int h = tid; h < nhdr; h += NT) hs[h] = hdr[dsc.hdr_off + h];
  const int r = tid;
  const bool row = r < nr;
  T* Sr = S + r;
  int h = 0, q0 = 0;
  while (h < nhdr) {
    // sweeps [h, h2) whose rotations fit in the chunk (a sweep has < n <= kRotChunk)
    __syncthreads();
    int h2 = h, tot = 0;
    while (h2 < nhdr && tot + hdr_count(hs[h2]) <= kRotChunk) tot += hdr_count(hs[h2++]);
    for (int q = tid; q < 2 * tot; q += NT) buf[q] = myrot[2 * q0 + q];
    __syncthreads();
    if (row) {
      const T* cs = buf;
      for (int hh = h; hh < h2; hh++) {
        const unsigned hw = hs[hh];
        const int start = hdr_start(hw), cnt = hdr_count(hw);
        const int dir = hdr_up(hw) ? -1 : 1;
        T carry = Sr[(size_t)(start + dir) * ld];
        int i = start;
        T v = Sr[(size_t)i * ld];
        for (int k = 0; k < cnt; k++) {
          const T c = cs[2 * k], sn = cs[2 * k + 1];
          const T vnext = (k + 1 < cnt) ? Sr[(size_t)(i - dir) * ld] : T(0);
          Sr[(size_t)(i + dir) * ld] = fma(c, carry, sn * v);
          carry = fma(c, v, -(sn * carry));
          v = vnext;
          i -= dir;
        }
        Sr[(size_t)(i + dir) * ld] = carry;
        cs += 2 * cnt;
      }
    }
    q0 += tot;
    h = h2;
  }
  __syncthreads();

  if (!done) {  // partial pass: write the rotated Q back for the next pass
    for (int j = 0; j < n; j++)
      for (int i = tid; i < nr; i += NT) Vg[(size_t)j * nr + i] = S[(size_t)j * ld + i];
    return;
  }

  // ---- sorteig!: stable ascending (isless order) ranks
  const T* dg = dg_all + dsc.w_off;
  for (int i = tid; i < n; i += NT) keys[i] = sort_key(dg[i]);
  __syncthreads();
  for (int i = tid; i < n; i += NT) {
    const unsigned long long ki = keys[i];
    int rk = 0;
    for (int j = 0; j < n; j++) {
      const unsigned long long kj = keys[j];
      rk += (kj < ki) || (kj == ki && j < i);
    }
    rank[i] = rk;
    const int se = scale_exp ? scale_exp[mid] : 0;
    T w = dg[i];
    if (se) w = (T)ldexp((double)w, se);
    wout[dsc.w_off + rk] = w;
  }
  __syncthreads();
  for (int j = 0; j < n; j++) {
    const int dst = rank[j];
    for (int i = tid; i < nr; i += NT) Vg[(size_t)dst * nr + i] = S[(size_t)j * ld + i];
  }
  if (tid == 0) cst[mid].applied = 1;
}

// Values-only runs (eigvalsPWK!): stable ascending sort of d into w.
template <class T>
__global__ void __launch_bounds__(128) k_sort_values(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                                     const T* __restrict__ dg_all, T* __restrict__ wout,
                                                     const int* __restrict__ info, const int* __restrict__ scale_exp) {
  __shared__ unsigned long long keys[kSmallMaxN];
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  const T* dg = dg_all + dsc.w_off;
  if (info[mid] == -1) {
    for (int i = tid; i < n; i += blockDim.x) wout[dsc.w_off + i] = (T)NAN;
    return;
  }
  for (int i = tid; i < n; i += blockDim.x) keys[i] = sort_key(dg[i]);
  __syncthreads();
  const int se = scale_exp ? scale_exp[mid] : 0;
  for (int i = tid; i < n; i += blockDim.x) {
    const unsigned long long ki = keys[i];
    int rk = 0;
    for (int j = 0; j < n; j++) rk += (keys[j] < ki) || (keys[j] == ki && j < i);
    T w = dg[i];
    if (se) w = (T)ldexp((double)w, se);
    wout[dsc.w_off + rk] = w;
  }
}


// SymTridiagonal input (eigen!(::SymTridiagonal), src/eigenSelfAdjoint.jl:602-612):
// d, e copied into the working arrays, Q := I, chase state reset.
template <class T>
__global__ void k_init_tridiagonal(const SmallDesc* __restrict__ descs, const int* __restrict__ perm,
                                   const T* __restrict__ din, const T* __restrict__ ein, T* __restrict__ d,
                                   T* __restrict__ e, T* __restrict__ Q, int* __restrict__ info,
                                   ChaseState* __restrict__ cst, bool wantq) {
  const int mid = perm[blockIdx.x];
  const SmallDesc dsc = descs[mid];
  const int n = dsc.n, tid = threadIdx.x;
  int bad = 0;
  for (int i = tid; i < n; i += blockDim.x) {
    const T di = din[dsc.w_off + i];
    const T ei = (i + 1 < n) ? ein[dsc.w_off + i] : T(0);
    bad |= !isfinite(di) || !isfinite(ei);
    d[dsc.w_off + i] = di;
    e[dsc.w_off + i] = ei;
  }
  bad = __syncthreads_or(bad);
  if (wantq)
    for (int idx = tid; idx < n * n; idx += blockDim.x) Q[dsc.a_off + idx] = (idx % (n + 1) == 0) ? T(1) : T(0);
  if (tid == 0) {
    ChaseState st;
    st.bs = 0;
    st.nsweeps = 0;
    st.nrot = 0;
    st.nhdr = 0;
    st.status = bad ? kChaseDone : kChaseRunning;
    st.applied = 0;
    cst[mid] = st;
    info[mid] = bad ? -1 : 0;
  }
}

cudaError_t apply_kernels_init() {
  cudaFuncSetAttribute(k_apply<double, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)apply_smem_bytes(kSmallMaxN, 8));
  cudaFuncSetAttribute(k_apply<float, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)apply_smem_bytes(kSmallMaxN, 4));
  cudaFuncSetAttribute(k_apply<double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)apply_smem_bytes(kSmallMaxN, 8));
  cudaFuncSetAttribute(k_apply<float, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       (int)apply_smem_bytes(kSmallMaxN, 4));
  return cudaGetLastError();
}

cudaError_t launch_apply(int tcode, int nblocks, int nt, size_t smem, cudaStream_t st, const SmallDesc* descs,
                         const int* perm, void* V, const void* d, void* w, ChaseState* cst, const void* rot,
                         const unsigned* hdr, const int* info, const int* scale_exp, bool rows2) {
  if (nblocks <= 0) return cudaSuccess;
#define GLA_AP(T, R2)                                                                                         \
  k_apply<T, R2><<<nblocks, nt, smem, st>>>(descs, perm, (T*)V, (const T*)d, (T*)w, cst, (const T*)rot, hdr, \
                                            info, scale_exp)
  if (tcode == kF64) {
    if (rows2) GLA_AP(double, true);
    else GLA_AP(double, false);
  } else {
    if (rows2) GLA_AP(float, true);
    else GLA_AP(float, false);
  }
#undef GLA_AP
  return cudaGetLastError();
}

cudaError_t launch_sort_values(int tcode, int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm,
                               const void* d, void* w, const int* info, const int* scale_exp) {
  if (nblocks <= 0) return cudaSuccess;
  if (tcode == kF64)
    k_sort_values<double><<<nblocks, 128, 0, st>>>(descs, perm, (const double*)d, (double*)w, info, scale_exp);
  else
    k_sort_values<float><<<nblocks, 128, 0, st>>>(descs, perm, (const float*)d, (float*)w, info, scale_exp);
  return cudaGetLastError();
}

__global__ void k_mark_unfinished(const SmallDesc* __restrict__ descs, const int* __restrict__ perm, int count,
                                  const ChaseState* __restrict__ cst, int* __restrict__ info) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int mid = perm[t];
  if (cst[mid].status != kChaseDone && info[mid] == 0) info[mid] = -2;
}

cudaError_t launch_mark_unfinished(int nblocks, cudaStream_t st, const SmallDesc* descs, const int* perm,
                                   const ChaseState* cst, int* info) {
  if (nblocks <= 0) return cudaSuccess;
  k_mark_unfinished<<<(nblocks + 127) / 128, 128, 0, st>>>(descs, perm, nblocks, cst, info);
  return cudaGetLastError();
}

cudaError_t launch_init_tridiagonal(int tcode, int nblocks, cudaStream_t st, const SmallDesc* descs,
                                    const int* perm, const void* din, const void* ein, void* d, void* e, void* Q,
                                    int* info, ChaseState* cst, bool wantq) {
  if (nblocks <= 0) return cudaSuccess;
  if (tcode == kF64)
    k_init_tridiagonal<double><<<nblocks, 128, 0, st>>>(descs, perm, (const double*)din, (const double*)ein,
                                                        (double*)d, (double*)e, (double*)Q, info, cst, wantq);
  else
    k_init_tridiagonal<float><<<nblocks, 128, 0, st>>>(descs, perm, (const float*)din, (const float*)ein,
                                                       (float*)d, (float*)e, (float*)Q, info, cst, wantq);
  return cudaGetLastError();
}

}  // namespace gla
