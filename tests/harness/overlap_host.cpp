// Host build of the operand aliasing test of the split-precision products
// (mref_overlap), for its CPU test: the same header the library includes.
#include <math.h>

#include "../../skkr_budapest_gb300/csrc/common.cuh"

// operands base + off (elements of one allocation), strides sk / sc, ld, the
// class map; returns mref_overlap for nk x nc items of `cols` columns
extern "C" int overlap_eval(long long offa, long long ska, long long sca, int lda, long long offb, long long skb,
                            long long scb, int ldb, const int *map, int nk, int nc, int cols) {
  static zd pool[1];
  MatRef a = mref_map(pool + offa, ska, sca, lda, map, nc);
  MatRef b = mref_map(pool + offb, skb, scb, ldb, map, nc);
  return mref_overlap(a, b, nk, nc, cols) ? 1 : 0;
}
