// Internal declarations shared by the small-matrix (n <= 128) batched
// eigensolver kernels and the host-side plan code.
#pragma once
#include <stdint.h>

#include "gla_common.cuh"

namespace gla {

constexpr int kSmallMaxN = 128;

// One entry per matrix of a batch, device resident.
struct SmallDesc {
  int n;
  int pad;
  long long a_off;    // element offset of the n x n column-major matrix in A / V
  long long w_off;    // element offset of its n eigenvalues (also of d, e)
  long long rot_off;  // offset, in rotations, of its rotation log
  long long hdr_off;  // offset, in headers, of its sweep-header log
  int rot_cap;        // rotation-log capacity per pass
  int hdr_cap;        // header-log capacity per pass
};

// Persistent chase state of one matrix between passes.
struct ChaseState {
  int bs;       // 0-based start of the active block
  int nsweeps;  // implicit-shift chases done so far
  int nrot;     // rotations logged in the current pass
  int nhdr;     // headers logged in the current pass
  int status;   // kChase* below
  int applied;  // apply kernel finished the matrix (sorted and written)
};
constexpr int kChaseRunning = 0;
constexpr int kChaseDone = 1;

// Sweep header: rotations start at column `start` and walk `count` columns
// down (QL: start, start-1, ...) or up (QR: start, start+1, ...).
GLA_DEV unsigned pack_hdr(int start, int count, int up) {
  return (unsigned)start | ((unsigned)count << 15) | ((unsigned)up << 30);
}
GLA_DEV int hdr_start(unsigned h) { return (int)(h & 0x7fff); }
GLA_DEV int hdr_count(unsigned h) { return (int)((h >> 15) & 0x7fff); }
GLA_DEV int hdr_up(unsigned h) { return (int)((h >> 30) & 1); }

// Order-preserving integer key of a float (isless order for non-NaN values:
// -0.0 sorts before +0.0).
GLA_DEV unsigned long long sort_key(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}
GLA_DEV unsigned long long sort_key(float x) {
  unsigned b = __float_as_uint(x);
  return (unsigned long long)((b >> 31) ? ~b : (b | 0x80000000u));
}

enum Algo { kAlgoQL = 0, kAlgoQR = 1, kAlgoPWK = 2 };

}  // namespace gla
