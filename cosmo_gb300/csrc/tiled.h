// Block-tiled copy of the stored FP32 matrix for the 8-vector product.
//
// Rows and columns are cut at the same boundaries (the neutron blocks of the
// basis: one neutron configuration followed by all its proton configurations;
// for a matrix read from a file, fixed 512-row ranges).  A tile is the nonzero
// part H[row block b, column block c]; the tiles of b are kept in ascending c.
// Inside a tile the entries are stored per 32-row slice of b, lane-interleaved
// (SELL-32: entry j of slice row l at run_start + 32 j + l, rows shorter than
// the slice's longest padded with value 0), each entry a 16-bit column inside
// block c and an FP32 value.  The product stages x[c] (contiguous rows) in
// shared memory with one bulk copy per tile, so every gather of the 8-vector
// row hits shared memory instead of L2.
#pragma once
#include "device.h"

namespace cg {

struct TiledOp {
  int nb = 0;                 // row (= column) blocks
  int lmax = 0;               // longest block
  int smax = 0;               // most 32-row slices in one block
  uint64_t ntiles = 0;        // nonzero (row block, column block) pairs
  uint64_t nruns = 0;         // (tile, slice) runs
  uint64_t entries = 0;       // stored entries including padding
  uint64_t nnz = 0;           // stored entries without padding
  int warps = 8, stages = 4;  // launch shape of the product
  DBuf<uint64_t> bstart;      // nb + 1
  DBuf<uint32_t> order;       // blocks, longest first
  DBuf<uint32_t> tptr;        // nb + 1: first tile of each block
  DBuf<uint32_t> tcb;         // per tile: column block
  DBuf<uint32_t> runbase;     // per block: first run; run of (tile t, slice s) = runbase + (t - tptr) * slices + s
  DBuf<uint32_t> roff;        // nruns + 1: first entry of each run / 32
  DBuf<uint16_t> col;         // entries: column inside the column block
  DBuf<float> val;            // entries: FP32 value (0 in padding)
  mutable DBuf<int> err;      // staged-copy / slot-release timeout flag
  uint64_t bytes() const {
    return bstart.bytes() + order.bytes() + tptr.bytes() + tcb.bytes() + runbase.bytes() + roff.bytes() +
           col.bytes() + val.bytes();
  }
};

// Longest block the product's shared-memory staging takes.
constexpr int kTiledMaxBlock = 2048;
// Shared memory ahead of the ring of staged x blocks (mbarriers, abort flag).
constexpr int kTiledHeadBytes = 128;

// Build h.tiled from the stored CSR FP32 values (h.hi) with the row/column
// blocks starting at bstart (nb + 1 entries, bstart[nb] = n).  Leaves h.tiled
// empty when a block is longer than kTiledMaxBlock.
void tiled_build(Hamiltonian& h, const std::vector<uint64_t>& bstart);
// Block starts used for a matrix without a basis: fixed 512-row ranges.
std::vector<uint64_t> tiled_uniform_blocks(uint64_t n);
// Y = H X for m <= 8 FP32 vectors; x rows are 8 floats (32 bytes, the
// buffer 16-byte aligned), only the first m outputs of each row are stored.
void tiled_product(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s);

}  // namespace cg
