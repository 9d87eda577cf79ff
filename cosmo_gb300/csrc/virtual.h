// On-the-fly ("virtual") H + lambda * J-J+ product: the matrix is never stored.
//
// Reference: SM::PPMatrix keeps the operator terms and applies them per bra
// (include/sm/PPMatrix.cxx:42-152: ReadDiagonal :191-211, TimesVectorSymmetric
// :117-152); DEXHVJT (davidson/DEXHVJT.cpp:36-78) drives Davidson with it.
//
// Here the product uses the proton-neutron product structure of the M-scheme
// basis.  Basis index = start(neutron block beta) + rank of the proton
// configuration inside the proton class complementary to beta, so every
// element of H belongs to one of these kinds (nu: neutron configuration,
// pi: proton configuration):
//   diagonal              D(nu, pi)
//   NN2  two neutrons move          h(nu -> nu')        x[nu', pi]   (same pi)
//   PP2  two protons move           h(pi -> pi')        x[nu, pi']   (same nu)
//   N1   one neutron moves, same m  c_n + s_n sum_{q in pi} Un[a][c][q]
//   P1   one proton moves, same m   c_p + s_p sum_{q in nu} Up[b][d][q]
//   NP   one neutron a->c and one proton b->d, m balanced:
//                                   s_n s_p W[a][c][b][d]      x[nu', pi']
// where s_n, s_p are the one-body fermion phases of each species (the phase of
// a proton-neutron two-body term factorises into them because neutrons precede
// protons in the s.p. order) and c_n / c_p hold the one-body term plus the
// same-species spectator terms.  The neutron transitions of each block and the
// proton transitions of each proton configuration (grouped by the change of
// 2m) are small host-built tables; the kernel walks them per row.
#pragma once
#include <cstdint>
#include <vector>

#include "device.h"

namespace cg {

struct NTrans {        // one neutron one-body transition of a block
  uint32_t target;     // target block
  uint8_t a, c;        // annihilated / created neutron s.p. index
  int8_t sign;         // 1: phase -1
  uint8_t dmi;         // slot: ((2m_c - 2m_a) / 2 + m2max) * 2 + parity change
  double cn;           // N1 value without the proton spectators (dmi == dm0 only)
};
static_assert(sizeof(NTrans) == 16, "NTrans layout");

struct VPair {         // NN2 (target block) / PP2 (target rank) element
  uint32_t target;
  uint32_t pad;
  double h;
};
static_assert(sizeof(VPair) == 16, "VPair layout");

struct VirtualOp {
  int nn = 0, np = 0, m2max = 0, ndm = 0, dm0 = 0;
  int nblocks = 0, lmax = 0;
  uint64_t nconf_p = 0;
  uint64_t connections = 0;  // generated elements per product (per vector)
  DBuf<uint64_t> bstart;                            // nblocks
  DBuf<uint32_t> blen, bclass, bmask, order;        // nblocks
  DBuf<uint32_t> cstart, cmask;                     // classes + 1, nconf_p
  DBuf<uint32_t> nt_off;                            // nblocks + 1
  DBuf<NTrans> nt;
  DBuf<uint32_t> nn_off;                            // nblocks + 1
  DBuf<VPair> nn2;
  // proton transitions and PP2 of each proton class in 32-row slices, lane-interleaved
  // (entry j of slice row l at off + 32 j + l, short lists padded with zero weights)
  DBuf<uint32_t> cslice;                            // nclasses + 1: first slice of each class
  DBuf<uint32_t> sl_off;                            // nslices * ndm + 1
  DBuf<uint32_t> sl_e;                              // rank | (b*np + d) << 16 | sign << 27
  DBuf<double> sl_c;                                // P1 value without neutron spectators
  DBuf<float> sl_cf;
  DBuf<uint32_t> pp_off;                            // nslices + 1
  DBuf<uint32_t> pp_rank;
  DBuf<double> pp_h;
  DBuf<float> pp_hf;
  DBuf<double> W, Un, Up;                           // nn*nn*np*np, nn*nn*np, np*np*nn
  DBuf<float> Wf, Unf, Upf;
  DBuf<float> Wl, Unl, Upl, sl_cl, pp_hl;            // low parts (value - float(value)), double-float product
  // truncated basis: rows of a block are a list (allowed proton configurations of its class);
  // proton-transition tables hold class ranks, mapped to list ranks by lmap (0xffff: outside)
  bool truncated = false;
  bool wide = false;                                // 64-bit species masks (bmask64, cmask64)
  DBuf<uint64_t> bmask64, cmask64;
  int rmax = 0;                                     // longest map (entries, a multiple of 8)
  DBuf<uint32_t> gcr;                               // nconf_p: class rank of each list member
  DBuf<uint16_t> lmap;                              // per list: class rank -> list rank
  DBuf<uint32_t> lmap_off, lmap_len;                // lists: first entry, entries (16-byte multiples)
  mutable DBuf<int> err;                            // staged-copy timeout flag
  uint64_t bytes() const {
    return bstart.bytes() + blen.bytes() + bclass.bytes() + bmask.bytes() + order.bytes() + cstart.bytes() +
           cmask.bytes() + nt_off.bytes() + nt.bytes() + nn_off.bytes() + nn2.bytes() + cslice.bytes() +
           sl_off.bytes() + sl_e.bytes() + sl_c.bytes() + sl_cf.bytes() + pp_off.bytes() + pp_rank.bytes() +
           pp_h.bytes() + pp_hf.bytes() + W.bytes() + Un.bytes() + Up.bytes() +
           Wf.bytes() + Unf.bytes() + Upf.bytes() + Wl.bytes() + Unl.bytes() + Upl.bytes() + sl_cl.bytes() +
           pp_hl.bytes() + gcr.bytes() + lmap.bytes() + lmap_off.bytes() + lmap_len.bytes() + bmask64.bytes() +
           cmask64.bytes();
  }
};

// Tables + diagonal for the on-the-fly product (h.diag filled, h.virt set).
void virtual_build(const System& sys, const Operator& op, const Basis& b, int precision, Hamiltonian& h);

// y[i*ldy + k] = (H x)[i][k], k < m, from x packed as n rows of kVirtualVB<T>
// values (zero-padded columns).  FP32: 8 vectors a row; FP64: 4.
void virtual_product_f32(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s);
void virtual_product_f64(const Hamiltonian& h, const double* x, double* y, int ldy, int m, cudaStream_t s);
// Double-float product (the refinement product): x packed by virtual_pack_df
// as n rows of 4 vectors in (hi, lo) FP32 pairs, y FP64, m <= 4; products and
// sums on the FP32 pipe, FP64-accurate to ~2^-44.
void virtual_product_df(const Hamiltonian& h, const float* x, double* y, int ldy, int m, cudaStream_t s);
void virtual_pack_df(uint64_t n, const double* x, int ld, int c0, int m, float* w, cudaStream_t s);
constexpr int kVirtualVB32 = 8, kVirtualVB64 = 4;
// pack columns c0 .. c0+m of a row-interleaved block into the product's layout
void virtual_pack_f32(uint64_t n, const float* x, int ld, int c0, int m, float* w, cudaStream_t s);
void virtual_pack_f64(uint64_t n, const double* x, int ld, int c0, int m, double* w, cudaStream_t s);
// general row-interleaved operands (any m, any ld); allocates its packing buffer
void virtual_launch(const Hamiltonian& h, int precision, const void* x, int ldx, void* y, int ldy, int m,
                    cudaStream_t s);

}  // namespace cg
