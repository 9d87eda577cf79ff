// Block-tiled copy of the stored FP32 matrix for the 8-vector product.
//
// Rows and columns are cut at the same boundaries (the neutron blocks of the
// basis: one neutron configuration followed by all its proton configurations;
// a matrix read from a .HH file has no basis and keeps the row-wise kernel).
// A tile is the nonzero part H[row block b, column block c]; the tiles of b
// are kept in ascending c.
// Inside a tile the entries are stored per 32-row slice of b, lane-interleaved
// (SELL-32: entry j of slice row l at run_start + 32 j + l, rows shorter than
// the slice's longest padded with value 0), each entry a 16-bit column inside
// block c and an FP32 value.  The product stages x[c] (contiguous rows) and
// the tile's entries (in chunks of at most gmax 32-entry groups) in shared
// memory with bulk copies, so every read of the inner loop hits shared memory.
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
  int rps = 1;                // 32-row slices per consumer warp
  int warps = 1, stages = 3;  // launch shape: consumer warps (= ceil(smax / rps)), ring slots
  DBuf<uint64_t> bstart;      // nb + 1
  DBuf<uint32_t> order;       // blocks, longest first
  DBuf<uint32_t> tptr;        // nb + 1: first tile of each block
  DBuf<uint32_t> tcb;         // per tile: column block
  DBuf<uint32_t> runbase;     // per block: first run; run of (tile t, slice s) = runbase + (t - tptr) * slices + s
  DBuf<uint32_t> roff;        // nruns + 1: first entry of each run / 32
  int gmax = 0;               // most 32-entry groups staged with one x block
  uint64_t nitems = 0;        // staged units (tile, group range)
  DBuf<uint32_t> iptr;        // nb + 1: first staged unit of each block
  DBuf<unsigned char> items;  // per unit: x rows, entry groups, run-offset copy (8 x u32)
  DBuf<uint32_t> rcopy;       // per tile: its run offsets, 16-byte aligned
  DBuf<uint32_t> dptr;        // nb + 1: first scaled-identity tile of each block
  DBuf<unsigned char> iden;   // per scaled-identity tile: first x row, value bits (2 x u32)
  uint64_t ident_tiles = 0, ident_nnz = 0;  // scaled-identity tiles and the entries they stand for
  DBuf<uint16_t> col;         // entries: column inside the column block
  DBuf<float> val;            // entries: FP32 value (0 in padding)
  mutable DBuf<int> err;      // staged-copy / slot-release timeout flag
  uint64_t bytes() const {
    return bstart.bytes() + order.bytes() + tptr.bytes() + tcb.bytes() + runbase.bytes() + roff.bytes() +
           iptr.bytes() + items.bytes() + rcopy.bytes() + dptr.bytes() + iden.bytes() + col.bytes() + val.bytes();
  }
};

// Stored entries from which an FP32 matrix built from a basis gets its tiled
// copy by default (below, the row-wise kernel is as fast and the copy is
// built on request, cg_spmm_set_format).
constexpr uint64_t kTiledMinEntries = uint64_t(1) << 26;
// Longest block the product's shared-memory staging takes.
constexpr int kTiledMaxBlock = 1536;
// Shared memory ahead of the ring of staged units (mbarriers, abort flag).
constexpr int kTiledHeadBytes = 128;
// Header of a ring slot: unit bounds (16 B) and the tile's run offsets (at
// most 60 u32: blocks of up to 59 slices).
constexpr int kTiledSlotHead = 256;

// Build h.tiled from the stored CSR FP32 values (h.hi) with the row/column
// blocks starting at bstart (nb + 1 entries, bstart[nb] = n).  Leaves h.tiled
// empty when a block is longer than kTiledMaxBlock.
void tiled_build(Hamiltonian& h, const std::vector<uint64_t>& bstart);
// Dynamic shared memory of the product with `stages` ring slots.
size_t tiled_smem(const TiledOp& t, int stages);
// Y = H X for m <= 8 FP32 vectors; x rows are 8 floats (32 bytes, the
// buffer 16-byte aligned), only the first m outputs of each row are stored.
void tiled_product(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s);

}  // namespace cg
