// Section table shared by the batched kernels: a batch is a list of
// independent sections (2-D or 3-D) packed one after another in the same
// flat, column-major arrays.
#pragma once

namespace pwd {

struct SecDesc {
  long off;       // element offset of the section in the input arrays
  long pout;      // element offset of its slopes in the output (2n for 3-D)
  long n;         // n1*n2*n3
  int n1, n2, n3;
  int tile0;      // first elementwise tile of the section
  int ntile;      // tiles of the section
  int ftile0;     // first column-strip tile (mixed-mode slope estimation)
  int nftile;     // column-strip tiles of the section
  int ctile0;     // first row-segment tile (mixed-mode slope estimation)
  int nctile;     // row-segment tiles of the section
  int gtile0;     // first axis-2 strip tile (mixed mode, cubes)
  int ngtile;     // axis-2 strip tiles of the section (0 unless n3 > 1)
  long line0[3];  // first global triangle line of each smoothed axis
  long scr0[3];   // triangle scratch offset of each smoothed axis
  long tr0;       // spray: first global trace (n2*n3 traces per section)
  long u0;        // spray: offset of the section's sprayed panels
  long sc0;       // spray: offset of the section's per-chain scratch
  long tp0;       // spray: first trace in the numbering padded to 32 per section
  int cord;       // spray: the section at this position of the padded numbering
};

// Section holding global item g, given each section's first item (sorted).
template <class F>
__device__ __forceinline__ int find_section(int nsec, long g, F first) {
  int lo = 0, hi = nsec - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (first(mid) <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

}  // namespace pwd
