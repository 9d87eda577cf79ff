// M-scheme basis on the GPU.
//
// The reference enumerates sorted N-tuples of s.p. indices in lexicographic
// order and keeps those with the wanted Jz, Tz and parity (SM::MakeMBS2,
// include/sm/MakeMBS.cxx:186-410, pruning at :290-296 is exact).  Because all
// neutron s.p. indices precede the proton ones
// (include/xsm/xSingleParticleStates.cxx:100-101), that order is: neutron
// configurations in lexicographic order, and inside each neutron block the
// proton configurations of the complementary (2m, parity) class, again in
// lexicographic order.  Here each species is a bitstring; the species
// configurations are unranked on the GPU, bucketed by class, and the
// proton x neutron product is expanded by one thread per basis state.
// The state index of any determinant is noff[colex(n)] + pcrank[colex(p)],
// which replaces the binary search of SM::locate
// (include/sm/ManyBodyStates.cxx:92-130).
#include <algorithm>
#include <map>

#include "device.h"

namespace cg {

Basis::~Basis() {
  if (stream) cudaStreamDestroy(stream);
}

namespace {

__global__ void k_unrank_lex(int norb, int k, uint64_t count, const uint64_t* __restrict__ binom,
                             const int* __restrict__ m2, const int* __restrict__ par, uint32_t* __restrict__ mask,
                             int* __restrict__ msum, int* __restrict__ psum) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  uint64_t r = i;
  uint32_t msk = 0;
  int ms = 0, ps = 0;
  int c = 0;
  for (int pos = 0; pos < k; ++pos) {
    // configurations whose pos-th element is c (given the prefix): C(norb-1-c, k-1-pos)
    for (;;) {
      if (c >= norb) return;  // only reachable for an out-of-range rank
      uint64_t cnt = binom[(norb - 1 - c) * kBinom + (k - 1 - pos)];
      if (r < cnt) break;
      r -= cnt;
      ++c;
    }
    msk |= 1u << c;
    ms += m2[c];
    ps ^= par[c];
    ++c;
  }
  mask[i] = msk;
  msum[i] = ms;
  psum[i] = ps;
}

// One thread per basis state: find the neutron block by binary search over the
// block starts, then pick the proton configuration from its class list.
__global__ void k_expand_product(uint64_t n, int nblocks, const uint64_t* __restrict__ bstart,
                                 const uint32_t* __restrict__ bmask, const uint32_t* __restrict__ bclass,
                                 const uint32_t* __restrict__ cstart, const uint32_t* __restrict__ cmasks, int nn,
                                 uint64_t* __restrict__ state) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nblocks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (bstart[mid] <= i) lo = mid; else hi = mid - 1;
  }
  uint64_t local = i - bstart[lo];
  uint32_t pm = cmasks[cstart[bclass[lo]] + local];
  state[i] = uint64_t(bmask[lo]) | (uint64_t(pm) << nn);
}

__global__ void k_tuples(uint64_t first, uint64_t count, int N, const uint64_t* __restrict__ state,
                         uint16_t* __restrict__ out) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  uint64_t s = state[first + i];
  uint16_t* o = out + i * N;
  int k = 0;
  while (s) {
    int b = __ffsll((long long)s) - 1;
    o[k++] = uint16_t(b);
    s &= s - 1;
  }
}

}  // namespace

uint64_t colex_host(uint64_t mask, const std::vector<uint64_t>& binom) {
  uint64_t r = 0;
  int i = 0;
  while (mask) {
    int c = __builtin_ctzll(mask);
    r += binom[c * kBinom + (i + 1)];
    ++i;
    mask &= mask - 1;
  }
  return r;
}

namespace {

void enumerate_species(SpeciesTables& sp, int norb, int k, const int* m2, const int* par, const DBuf<uint64_t>& binom,
                       const std::vector<uint64_t>& hb, cudaStream_t s) {
  sp.norb = norb;
  sp.k = k;
  sp.nconf = (k <= norb) ? hb[norb * kBinom + k] : 0;
  if (sp.nconf > (1ull << 30)) throw Error(CG_ERR_UNSUPPORTED, "species configuration space too large");
  sp.lex_mask.assign(sp.nconf, 0);
  sp.lex_m2.assign(sp.nconf, 0);
  sp.lex_par.assign(sp.nconf, 0);
  if (!sp.nconf) return;
  DBuf<int> dm2(norb > 0 ? norb : 1), dpar(norb > 0 ? norb : 1);
  if (norb) {
    dm2.upload(m2, norb, s);
    dpar.upload(par, norb, s);
  }
  DBuf<uint32_t> dmask(sp.nconf);
  DBuf<int> dms(sp.nconf), dps(sp.nconf);
  int T = 256;
  k_unrank_lex<<<unsigned((sp.nconf + T - 1) / T), T, 0, s>>>(norb, k, sp.nconf, binom.p, dm2.p, dpar.p, dmask.p,
                                                               dms.p, dps.p);
  CG_CUDA(cudaGetLastError());
    count_launch();
  CG_CUDA(cudaMemcpyAsync(sp.lex_mask.data(), dmask.p, sp.nconf * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaMemcpyAsync(sp.lex_m2.data(), dms.p, sp.nconf * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaMemcpyAsync(sp.lex_par.data(), dps.p, sp.nconf * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void basis_build(const System& sys, Basis& b) {
  if (sys.n_neutron_states > 32 || int(sys.sps.size()) - sys.n_neutron_states > 32) {
    basis_build_wide(sys, b);
    return;
  }
  CG_CUDA(cudaGetDevice(&b.device));
  if (!b.stream) CG_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
  cudaStream_t s = b.stream;
  b.ns = int(sys.sps.size());
  b.nn = sys.n_neutron_states;
  b.np = b.ns - b.nn;
  b.kn = sys.nv;
  b.kp = sys.zv;
  b.twom = sys.twom;
  b.parity = sys.parity;
  if (b.nn > 32 || b.np > 32) throw Error(CG_ERR_UNSUPPORTED, "more than 32 m-states per species");
  b.sp_m2.resize(b.ns);
  b.sp_par.resize(b.ns);
  for (int i = 0; i < b.ns; ++i) {
    b.sp_m2[i] = sys.sps[i].m2;
    b.sp_par[i] = sys.sps[i].parity;
  }
  b.h_binom.assign(kBinom * kBinom, 0);
  for (int a = 0; a < kBinom; ++a) {
    b.h_binom[a * kBinom] = 1;
    for (int c = 1; c <= a; ++c) b.h_binom[a * kBinom + c] = b.h_binom[(a - 1) * kBinom + c - 1] + (c <= a - 1 ? b.h_binom[(a - 1) * kBinom + c] : 0);
  }
  b.binom.alloc(kBinom * kBinom);
  b.binom.upload(b.h_binom, s);

  enumerate_species(b.neut, b.nn, b.kn, b.sp_m2.data(), b.sp_par.data(), b.binom, b.h_binom, s);
  enumerate_species(b.prot, b.np, b.kp, b.sp_m2.data() + b.nn, b.sp_par.data() + b.nn, b.binom, b.h_binom, s);

  // proton classes keyed by (2m, parity), each in lexicographic order
  std::map<std::pair<int, int>, std::vector<uint32_t>> cls;
  for (uint64_t i = 0; i < b.prot.nconf; ++i) cls[{b.prot.lex_m2[i], b.prot.lex_par[i]}].push_back(uint32_t(i));
  std::map<std::pair<int, int>, uint32_t> cls_id;
  std::vector<uint32_t> cstart, cmasks;
  b.h_pcrank.assign(std::max<uint64_t>(b.prot.nconf, 1), 0);
  for (auto& kv : cls) {
    cls_id[kv.first] = uint32_t(cstart.size());
    cstart.push_back(uint32_t(cmasks.size()));
    uint32_t r = 0;
    for (uint32_t li : kv.second) {
      uint32_t pm = b.prot.lex_mask[li];
      cmasks.push_back(pm);
      b.h_pcrank[colex_host(pm, b.h_binom)] = r++;
    }
  }
  // neutron blocks in lexicographic order
  b.h_noff.assign(std::max<uint64_t>(b.neut.nconf, 1), ~0ull);
  std::vector<uint64_t> bstart;
  std::vector<uint32_t> bmask, bclass;
  uint64_t off = 0;
  const Truncation& tr = sys.trunc;
  b.truncated = tr.active();
  if (!b.truncated) {
    for (uint64_t i = 0; i < b.neut.nconf; ++i) {
      auto it = cls_id.find({b.twom - b.neut.lex_m2[i], b.parity ^ b.neut.lex_par[i]});
      if (it == cls_id.end()) continue;
      uint64_t cnt = cls[{b.twom - b.neut.lex_m2[i], b.parity ^ b.neut.lex_par[i]}].size();
      uint32_t nm = b.neut.lex_mask[i];
      b.h_noff[colex_host(nm, b.h_binom)] = off;
      bstart.push_back(off);
      bmask.push_back(nm);
      bclass.push_back(it->second);
      off += cnt;
    }
  } else {
    // the truncated basis keeps the untruncated order (XsysmbsOMP writes its
    // determinants from a sorted map, xmlshell/xmbs/XsysmbsOMP.cpp:405-428):
    // neutron configurations in lexicographic order, each followed by the
    // allowed proton configurations of its class in lexicographic order
    const int R = int(tr.rejections.size());
    std::vector<int> q(b.ns);
    for (int i = 0; i < b.ns; ++i) q[i] = sp_quanta(sys.sps[i]);
    int ncore = 0, pcore = 0;  // SM::CoreQuanta: the first Nv (Zv) s.p. states in list order
    for (int i = 0; i < std::min(b.kn, b.nn); ++i) ncore += q[i];
    for (int i = 0; i < std::min(b.kp, b.np); ++i) pcore += q[b.nn + i];
    auto quanta = [&](uint64_t gmask) {
      int Q = 0;
      for (uint64_t m = gmask; m; m &= m - 1) Q += q[__builtin_ctzll(m)];
      return Q;
    };
    // per proton configuration (lexicographic index): quanta above the core and rejection counts
    std::vector<int> pq(b.prot.nconf), pc(b.prot.nconf * std::max(R, 1));
    for (uint64_t i = 0; i < b.prot.nconf; ++i) {
      const uint64_t gm = uint64_t(b.prot.lex_mask[i]) << b.nn;
      pq[i] = quanta(gm) - pcore;
      for (int r = 0; r < R; ++r) pc[i * R + r] = __builtin_popcountll(gm & tr.rejections[r].mask);
    }
    // lexicographic index of each proton class member (cls holds them in rank order)
    std::map<std::vector<int>, uint32_t> list_id;
    std::vector<std::vector<uint32_t>> lists;  // lexicographic proton indices
    b.npc = b.prot.nconf;
    b.h_nlist.assign(std::max<uint64_t>(b.neut.nconf, 1), ~0u);
    for (uint64_t i = 0; i < b.neut.nconf; ++i) {
      const std::pair<int, int> ckey{b.twom - b.neut.lex_m2[i], b.parity ^ b.neut.lex_par[i]};
      auto it = cls_id.find(ckey);
      if (it == cls_id.end()) continue;
      const uint64_t gm = b.neut.lex_mask[i];
      const int qn = quanta(gm) - ncore;
      if (tr.hw && (qn < 0 || qn > tr.hwmax)) continue;
      std::vector<int> key{int(it->second), qn};
      for (int r = 0; r < R; ++r) key.push_back(__builtin_popcountll(gm & tr.rejections[r].mask));
      auto lit = list_id.find(key);
      if (lit == list_id.end()) {
        std::vector<uint32_t> keep;
        for (uint32_t li : cls[ckey]) {
          const int qp = pq[li];
          if (tr.hw && (qp < 0 || qp > tr.hwmax || qn + qp < tr.hwmin || qn + qp > tr.hwmax)) continue;
          bool ok = true;
          for (int r = 0; r < R && ok; ++r) {
            const int c = key[2 + r] + pc[li * R + r];
            ok = c >= tr.rejections[r].nmin && c <= tr.rejections[r].nmax;
          }
          if (ok) keep.push_back(li);
        }
        lit = list_id.emplace(key, uint32_t(lists.size())).first;
        lists.push_back(std::move(keep));
      }
      const std::vector<uint32_t>& lst = lists[lit->second];
      if (lst.empty()) continue;
      const uint32_t nm = b.neut.lex_mask[i];
      const uint64_t cn = colex_host(nm, b.h_binom);
      b.h_noff[cn] = off;
      b.h_nlist[cn] = lit->second;
      bstart.push_back(off);
      bmask.push_back(nm);
      bclass.push_back(lit->second);
      off += lst.size();
    }
    // the lists take the place of the classes; per-list ranks by proton colex rank
    cstart.clear();
    cmasks.clear();
    b.h_lrank.assign(std::max<uint64_t>(lists.size() * b.npc, 1), ~0u);
    for (size_t L = 0; L < lists.size(); ++L) {
      cstart.push_back(uint32_t(cmasks.size()));
      uint32_t r = 0;
      for (uint32_t li : lists[L]) {
        const uint32_t pm = b.prot.lex_mask[li];
        cmasks.push_back(pm);
        b.h_lrank[L * b.npc + colex_host(pm, b.h_binom)] = r++;
      }
    }
    b.nlist.upload(b.h_nlist, s);
    b.lrank.upload(b.h_lrank, s);
  }
  b.n = off;
  cstart.push_back(uint32_t(cmasks.size()));
  b.h_bstart = bstart;
  b.h_bmask = bmask;
  b.h_bclass = bclass;
  b.h_cstart = cstart;
  b.h_cmasks = cmasks;
  b.noff.upload(b.h_noff, s);
  b.pcrank.upload(b.h_pcrank, s);
  b.state.alloc(std::max<uint64_t>(b.n, 1));
  if (b.n) {
    DBuf<uint64_t> dbs;
    DBuf<uint32_t> dbm, dbc, dcs, dcm;
    dbs.upload(bstart, s);
    dbm.upload(bmask, s);
    dbc.upload(bclass, s);
    dcs.upload(cstart, s);
    dcm.upload(cmasks, s);
    int T = 256;
    k_expand_product<<<unsigned((b.n + T - 1) / T), T, 0, s>>>(b.n, int(bstart.size()), dbs.p, dbm.p, dbc.p, dcs.p,
                                                                dcm.p, b.nn, b.state.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));
  }
}

void basis_tuples(const Basis& b, uint64_t first, uint64_t count, uint16_t* out) {
  if (first + count > b.n) throw Error(CG_ERR_ARG, "state range outside the basis");
  if (b.wide) {
    basis_tuples_wide(b, first, count, out);
    return;
  }
  int N = b.kn + b.kp;
  const uint64_t chunk = 1ull << 24;
  DBuf<uint16_t> d(std::min(count, chunk) * std::max(N, 1));
  for (uint64_t c0 = 0; c0 < count; c0 += chunk) {
    uint64_t c = std::min(chunk, count - c0);
    int T = 256;
    k_tuples<<<unsigned((c + T - 1) / T), T, 0, b.stream>>>(first + c0, c, N, b.state.p, d.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaMemcpyAsync(out + c0 * N, d.p, c * N * sizeof(uint16_t), cudaMemcpyDeviceToHost, b.stream));
    CG_CUDA(cudaStreamSynchronize(b.stream));
  }
}

uint64_t basis_locate_host(const Basis& b, const uint16_t* t) {
  if (b.wide) return basis_locate_wide_host(b, t);
  const uint64_t miss = b.n + 1;
  int N = b.kn + b.kp;
  uint64_t nmask = 0, pmask = 0;
  int kn = 0, kp = 0, m2n = 0, m2p = 0, pn = 0, pp = 0;
  for (int i = 0; i < N; ++i) {
    if (i && t[i] <= t[i - 1]) return miss;
    int x = t[i];
    if (x >= b.ns) return miss;
    if (x < b.nn) { nmask |= 1ull << x; ++kn; m2n += b.sp_m2[x]; pn ^= b.sp_par[x]; }
    else { pmask |= 1ull << (x - b.nn); ++kp; m2p += b.sp_m2[x]; pp ^= b.sp_par[x]; }
  }
  if (kn != b.kn || kp != b.kp || m2n + m2p != b.twom || (pn ^ pp) != b.parity) return miss;
  const uint64_t cn = colex_host(nmask, b.h_binom);
  uint64_t no = b.h_noff[cn];
  if (no == ~0ull) return miss;
  if (b.truncated) {
    const uint32_t r = b.h_lrank[uint64_t(b.h_nlist[cn]) * b.npc + colex_host(pmask, b.h_binom)];
    return r == ~0u ? miss : no + r;
  }
  return no + b.h_pcrank[colex_host(pmask, b.h_binom)];
}

}  // namespace cg
