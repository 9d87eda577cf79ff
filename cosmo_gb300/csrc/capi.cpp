// extern "C" entry points of libcosmo_gb300: status codes in, exceptions never
// out.  Each call maps to one reference interface (see include/cosmo_gb300.h).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <string>

#include "cosmo_gb300.h"
#include "davidson.h"
#include "dense.h"
#include "device.h"
#include "model.h"
#include "batched.h"
#include "tiled.h"
#include "virtual.h"
#include "xshljt.h"

struct cg_problem {
  cg::System sys;
  cg::Operator op;
};
struct cg_basis {
  cg::Basis b;
  cg::System sys;
};
struct cg_hamiltonian {
  cg::Hamiltonian h;
};
struct cg_batch {
  cg::BatchSet bs;
};

namespace {
thread_local std::string g_err;

template <class F>
cg_status guard(F&& f) {
  try {
    g_err.clear();
    f();
    return CG_OK;
  } catch (const cg::Error& e) {
    g_err = e.what();
    return e.code;
  } catch (const std::bad_alloc&) {
    g_err = "host allocation failed";
    return CG_ERR_NOMEM;
  } catch (const std::exception& e) {
    g_err = e.what();
    return CG_ERR_INTERNAL;
  } catch (...) {
    g_err = "unknown error";
    return CG_ERR_INTERNAL;
  }
}

void require_device() {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess || n == 0)
    throw cg::Error(CG_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
}

void same_device(int dev) {
  int cur = -1;
  CG_CUDA(cudaGetDevice(&cur));
  if (cur != dev) throw cg::Error(CG_ERR_ARG, "handle belongs to another CUDA device; make it current first");
}

#define CG_NOT_NULL(p) \
  if (!(p)) throw cg::Error(CG_ERR_ARG, #p " is NULL")
}  // namespace

namespace cg {
uint64_t& launch_counter() {
  static uint64_t c = 0;
  return c;
}
}  // namespace cg

extern "C" {

const char* cg_last_error(void) { return g_err.c_str(); }
uint64_t cg_launch_count(void) { return cg::launch_counter(); }
int32_t cg_version(void) { return 100; }
int32_t cg_device_count(void) {
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    g_err = cudaGetErrorString(e);
    return e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver ? 0 : CG_ERR_CUDA;
  }
  return n;
}

// ------------------------------------------------------------- problem
cg_status cg_problem_load_xml(const char* xml_path, const char* system_name, cg_problem** out) {
  return guard([&] {
    CG_NOT_NULL(xml_path);
    CG_NOT_NULL(out);
    *out = nullptr;
    auto p = std::make_unique<cg_problem>();
    p->sys = cg::load_system(xml_path, system_name ? system_name : "");
    p->op = cg::build_operator(p->sys);
    *out = p.release();
  });
}
cg_status cg_problem_create(const cg_problem_desc* d, cg_problem** out) {
  return guard([&] {
    CG_NOT_NULL(d);
    CG_NOT_NULL(out);
    *out = nullptr;
    if (d->n_sps < 1 || d->n_neutron_sps < 0 || d->n_neutron_sps > d->n_sps)
      throw cg::Error(CG_ERR_ARG, "bad s.p. table size");
    if (d->n_neutron_sps > 64 || d->n_sps - d->n_neutron_sps > 64)
      throw cg::Error(CG_ERR_UNSUPPORTED, "more than 64 m-scheme s.p. states per species");
    CG_NOT_NULL(d->sps);
    if (d->nv < 0 || d->zv < 0) throw cg::Error(CG_ERR_ARG, "negative particle number");
    auto p = std::make_unique<cg_problem>();
    cg::System& s = p->sys;
    s.name = "terms";
    s.nv = d->nv;
    s.zv = d->zv;
    s.twom = d->twom;
    s.parity = d->parity & 1;
    s.n_neutron_states = d->n_neutron_sps;
    for (int i = 0; i < d->n_sps; ++i) {
      const int32_t* r = d->sps + 8 * i;
      cg::SPState x{r[0], r[1], r[2], r[3], r[4], r[5], r[6], r[7]};
      bool neutron = i < d->n_neutron_sps;
      if ((neutron && x.tz2 != 1) || (!neutron && x.tz2 != -1))
        throw cg::Error(CG_ERR_ARG, "s.p. table must list neutrons (2tz=+1) before protons (2tz=-1)");
      s.sps.push_back(x);
    }
    auto key_ok = [&](int k) { return k >= 0 && k < d->n_sps; };
    if (d->n_one_body) { CG_NOT_NULL(d->one_keys); CG_NOT_NULL(d->one_vals); }
    if (d->n_two_body) { CG_NOT_NULL(d->two_keys); CG_NOT_NULL(d->two_vals); }
    for (int64_t k = 0; k < d->n_one_body; ++k) {
      int a = d->one_keys[2 * k], b = d->one_keys[2 * k + 1];
      if (!key_ok(a) || !key_ok(b) || b < a) throw cg::Error(CG_ERR_ARG, "one-body key out of range or not forward");
      p->op.one[{a, b}] += d->one_vals[k];
    }
    for (int64_t k = 0; k < d->n_two_body; ++k) {
      const int32_t* q = d->two_keys + 4 * k;
      for (int j = 0; j < 4; ++j)
        if (!key_ok(q[j])) throw cg::Error(CG_ERR_ARG, "two-body key out of range");
      bool fwd = q[0] <= q[1] && q[2] <= q[3] && (q[0] < q[2] || (q[0] == q[2] && q[1] <= q[3]));
      if (!fwd) throw cg::Error(CG_ERR_ARG, "two-body key is not forward ordered");
      p->op.two[{q[0], q[1], q[2], q[3]}] += d->two_vals[k];
    }
    *out = p.release();
  });
}

void cg_problem_destroy(cg_problem* p) { delete p; }

cg_status cg_problem_get_info(const cg_problem* p, cg_problem_info* info) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(info);
    info->n_sps = int32_t(p->sys.sps.size());
    info->n_neutron_sps = p->sys.n_neutron_states;
    info->nv = p->sys.nv;
    info->zv = p->sys.zv;
    info->twom = p->sys.twom;
    info->parity = p->sys.parity;
    info->has_jj = p->sys.has_jj;
    info->jj = p->sys.jj;
    info->n_one_body = int64_t(p->op.one.size());
    info->n_two_body = int64_t(p->op.two.size());
  });
}

cg_status cg_problem_sps(const cg_problem* p, int32_t* t) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(t);
    for (size_t i = 0; i < p->sys.sps.size(); ++i) {
      const auto& s = p->sys.sps[i];
      int32_t* r = t + 8 * i;
      r[0] = s.level; r[1] = s.n; r[2] = s.l; r[3] = s.j2; r[4] = s.m2; r[5] = s.t2; r[6] = s.tz2; r[7] = s.parity;
    }
  });
}

cg_status cg_problem_one_body(const cg_problem* p, int32_t* keys, double* vals) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(keys);
    CG_NOT_NULL(vals);
    size_t k = 0;
    for (auto& kv : p->op.one) {
      keys[2 * k] = kv.first[0];
      keys[2 * k + 1] = kv.first[1];
      vals[k++] = kv.second;
    }
  });
}

cg_status cg_problem_two_body(const cg_problem* p, int32_t* keys, double* vals) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(keys);
    CG_NOT_NULL(vals);
    size_t k = 0;
    for (auto& kv : p->op.two) {
      for (int j = 0; j < 4; ++j) keys[4 * k + j] = kv.first[j];
      vals[k++] = kv.second;
    }
  });
}

// ---------------------------------------------------------------- basis
cg_status cg_basis_build(const cg_problem* p, cg_basis** out) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(out);
    *out = nullptr;
    require_device();
    auto b = std::make_unique<cg_basis>();
    b->sys = p->sys;
    cg::basis_build(p->sys, b->b);
    *out = b.release();
  });
}
cg_status cg_basis_build_wide(const cg_problem* p, cg_basis** out) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(out);
    *out = nullptr;
    require_device();
    auto b = std::make_unique<cg_basis>();
    b->sys = p->sys;
    cg::basis_build_wide(p->sys, b->b);
    *out = b.release();
  });
}
cg_status cg_basis_is_wide(const cg_basis* b, int32_t* wide) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(wide);
    *wide = b->b.wide ? 1 : 0;
  });
}
void cg_basis_destroy(cg_basis* b) { delete b; }

cg_status cg_basis_dims(const cg_basis* b, uint64_t* n, int32_t* np) {
  return guard([&] {
    CG_NOT_NULL(b);
    if (n) *n = b->b.n;
    if (np) *np = b->b.kn + b->b.kp;
  });
}

cg_status cg_basis_states(const cg_basis* b, uint64_t first, uint64_t count, uint16_t* tuples) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(tuples);
    same_device(b->b.device);
    cg::basis_tuples(b->b, first, count, tuples);
  });
}

cg_status cg_basis_locate(const cg_basis* b, const uint16_t* tuples, uint64_t count, uint64_t* out) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(tuples);
    CG_NOT_NULL(out);
    int N = b->b.kn + b->b.kp;
    for (uint64_t k = 0; k < count; ++k) out[k] = cg::basis_locate_host(b->b, tuples + k * N);
  });
}

cg_status cg_basis_write_mbs(const cg_basis* b, const char* path) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(path);
    same_device(b->b.device);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw cg::Error(CG_ERR_IO, std::string("cannot write ") + path);
    int32_t N = b->b.kn + b->b.kp;
    uint64_t n = b->b.n;
    f.write(reinterpret_cast<const char*>(&N), 4);
    f.write(reinterpret_cast<const char*>(&n), 8);
    const uint64_t chunk = 1ull << 22;
    std::vector<uint16_t> buf;
    for (uint64_t s = 0; s < n; s += chunk) {
      uint64_t c = std::min(chunk, n - s);
      buf.resize(c * N);
      cg::basis_tuples(b->b, s, c, buf.data());
      f.write(reinterpret_cast<const char*>(buf.data()), c * N * 2);
    }
    if (!f) throw cg::Error(CG_ERR_IO, std::string("write failed: ") + path);
  });
}

// ---------------------------------------------------------- Hamiltonian
cg_status cg_hamiltonian_build(const cg_problem* p, const cg_basis* b, int32_t precision, cg_hamiltonian** out) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(b);
    CG_NOT_NULL(out);
    *out = nullptr;
    same_device(b->b.device);
    if (p->sys.sps.size() != b->sys.sps.size() || p->sys.nv != b->sys.nv || p->sys.zv != b->sys.zv)
      throw cg::Error(CG_ERR_ARG, "basis was built for another problem");
    auto h = std::make_unique<cg_hamiltonian>();
    cg::hamiltonian_build(p->sys, p->op, b->b, precision, h->h);
    *out = h.release();
  });
}
cg_status cg_hamiltonian_build_virtual(const cg_problem* p, const cg_basis* b, int32_t precision,
                                       cg_hamiltonian** out) {
  return guard([&] {
    CG_NOT_NULL(p);
    CG_NOT_NULL(b);
    CG_NOT_NULL(out);
    *out = nullptr;
    same_device(b->b.device);
    if (p->sys.sps.size() != b->sys.sps.size() || p->sys.nv != b->sys.nv || p->sys.zv != b->sys.zv)
      throw cg::Error(CG_ERR_ARG, "basis was built for another problem");
    auto h = std::make_unique<cg_hamiltonian>();
    cg::virtual_build(p->sys, p->op, b->b, precision, h->h);
    *out = h.release();
  });
}

cg_status cg_hamiltonian_is_virtual(const cg_hamiltonian* h, int32_t* is_virtual) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(is_virtual);
    *is_virtual = h->h.virt ? 1 : 0;
  });
}

void cg_hamiltonian_destroy(cg_hamiltonian* h) { delete h; }

cg_status cg_hamiltonian_get_info(const cg_hamiltonian* h, cg_hamiltonian_info* info) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(info);
    info->n = h->h.n;
    info->nnz_full = h->h.nnz;
    info->nnz_upper = h->h.nnz_upper;
    info->precision = h->h.precision;
    info->max_row = h->h.max_row;
    info->device_bytes = h->h.device_bytes();
    info->build_seconds = h->h.build_seconds;
  });
}

cg_status cg_hamiltonian_diagonal(const cg_hamiltonian* h, double* d) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(d);
    same_device(h->h.device);
    CG_CUDA(cudaMemcpy(d, h->h.diag.p, h->h.n * 8, cudaMemcpyDeviceToHost));
  });
}

cg_status cg_hamiltonian_upper_rows(const cg_hamiltonian* h, uint64_t row0, uint64_t nrows, uint64_t* rowptr,
                                    uint32_t* cols, double* vals) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(rowptr);
    same_device(h->h.device);
    if (h->h.virt) throw cg::Error(CG_ERR_UNSUPPORTED, "an on-the-fly Hamiltonian stores no rows");
    cg::hamiltonian_upper_rows(h->h, row0, nrows, rowptr, cols, vals);
  });
}

cg_status cg_hamiltonian_write_hh(const cg_hamiltonian* h, const char* path) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(path);
    same_device(h->h.device);
    if (h->h.virt) throw cg::Error(CG_ERR_UNSUPPORTED, "an on-the-fly Hamiltonian stores no rows");
    std::ofstream f(path, std::ios::binary);
    if (!f) throw cg::Error(CG_ERR_IO, std::string("cannot write ") + path);
    uint64_t n = h->h.n;
    f.write(reinterpret_cast<const char*>(&n), 8);
    const uint64_t chunk = 1 << 16;
    for (uint64_t r0 = 0; r0 < n; r0 += chunk) {
      uint64_t nr = std::min(chunk, n - r0);
      std::vector<uint64_t> rp(nr + 1);
      cg::hamiltonian_upper_rows(h->h, r0, nr, rp.data(), nullptr, nullptr);
      std::vector<uint32_t> c(rp[nr]);
      std::vector<double> v(rp[nr]);
      cg::hamiltonian_upper_rows(h->h, r0, nr, rp.data(), c.data(), v.data());
      for (uint64_t r = 0; r < nr; ++r) {
        uint32_t nz = uint32_t(rp[r + 1] - rp[r]);
        f.write(reinterpret_cast<const char*>(&nz), 4);
        for (uint64_t k = rp[r]; k < rp[r + 1]; ++k) {
          uint64_t ind = c[k];
          f.write(reinterpret_cast<const char*>(&ind), 8);
        }
        f.write(reinterpret_cast<const char*>(v.data() + rp[r]), 8 * nz);
      }
    }
    if (!f) throw cg::Error(CG_ERR_IO, std::string("write failed: ") + path);
  });
}

cg_status cg_hamiltonian_read_hh(const char* path, int32_t precision, cg_hamiltonian** out) {
  return guard([&] {
    CG_NOT_NULL(path);
    CG_NOT_NULL(out);
    *out = nullptr;
    require_device();
    auto h = std::make_unique<cg_hamiltonian>();
    cg::hamiltonian_read_hh(path, precision, h->h);
    *out = h.release();
  });
}

void* cg_hamiltonian_stream(const cg_hamiltonian* h) { return h ? static_cast<void*>(h->h.stream) : nullptr; }

// ------------------------------------------------------------------ SpMM
cg_status cg_spmm(const cg_hamiltonian* h, const double* x, double* y, int32_t m, int32_t precision) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(x);
    CG_NOT_NULL(y);
    same_device(h->h.device);
    cg::spmm_host(h->h, precision, x, y, m);
  });
}

cg_status cg_spmm_device(const cg_hamiltonian* h, const void* x, int32_t ldx, void* y, int32_t ldy, int32_t m,
                         int32_t precision) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(x);
    CG_NOT_NULL(y);
    same_device(h->h.device);
    cg::spmm_launch(h->h, precision, x, ldx, y, ldy, m, h->h.stream);
  });
}

cg_status cg_spmm_autotune(cg_hamiltonian* h, int32_t nvec, int32_t reps, int32_t* n_candidates, int32_t* warps,
                           int32_t* ctas_per_sm, float* ms) {
  return guard([&] {
    CG_NOT_NULL(h);
    same_device(h->h.device);
    if (nvec < 1 || nvec > 16) throw cg::Error(CG_ERR_ARG, "nvec must be in 1..16");
    auto c = cg::spmm_autotune(h->h, nvec, std::max(1, reps));
    if (n_candidates) {
      int cap = *n_candidates;
      for (int i = 0; i < int(c.size()) && i < cap; ++i) {
        if (warps) warps[i] = c[i].warps;
        if (ctas_per_sm) ctas_per_sm[i] = c[i].ctas_per_sm;
        if (ms) ms[i] = c[i].ms;
      }
      *n_candidates = int(c.size());
    }
  });
}

cg_status cg_spmm_refine_static(const cg_hamiltonian* h, const double* x, int32_t ldx, double* y, int32_t ldy,
                                int32_t m) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(x);
    CG_NOT_NULL(y);
    same_device(h->h.device);
    cg::spmm_refine_static(h->h, x, ldx, y, ldy, m, h->h.stream);
  });
}

cg_status cg_spmm_refine_static_max_rows(uint64_t* rows) {
  return guard([&] {
    CG_NOT_NULL(rows);
    *rows = cg::spmm_refine_static_max_rows();
  });
}

cg_status cg_batch_create(const cg_problem* const* problems, int32_t count, cg_batch** out) {
  return guard([&] {
    CG_NOT_NULL(problems);
    CG_NOT_NULL(out);
    *out = nullptr;
    if (count < 1) throw cg::Error(CG_ERR_ARG, "count must be >= 1");
    std::vector<const cg::System*> sys;
    std::vector<const cg::Operator*> ops;
    for (int i = 0; i < count; ++i) {
      CG_NOT_NULL(problems[i]);
      sys.push_back(&problems[i]->sys);
      ops.push_back(&problems[i]->op);
    }
    require_device();
    auto b = std::make_unique<cg_batch>();
    cg::batch_build(sys, ops, b->bs);
    *out = b.release();
  });
}

void cg_batch_destroy(cg_batch* b) { delete b; }

cg_status cg_batch_defaults(cg_batch_params* prm) {
  return guard([&] {
    CG_NOT_NULL(prm);
    cg::BatchParams d;
    prm->nstates = d.nev;
    prm->block = d.block;
    prm->lim = d.lim;
    prm->keep = d.keep;
    prm->maxiter = d.maxiter;
    prm->tol_resid = d.tol_resid;
    prm->switch_resid = d.switch_resid;
    prm->use_graph = d.use_graph ? 1 : 0;
  });
}

cg_status cg_batch_dims(const cg_batch* b, uint64_t* dims) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(dims);
    for (int p = 0; p < b->bs.np; ++p) dims[p] = b->bs.dims[p];
  });
}

cg_status cg_batch_solve(cg_batch* b, const cg_batch_params* prm, double* eig, double* resid, int32_t* nconv,
                         cg_batch_stats* stats) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(prm);
    CG_NOT_NULL(eig);
    same_device(b->bs.device);
    cg::BatchParams p;
    p.nev = prm->nstates;
    p.block = prm->block;
    p.lim = prm->lim;
    p.keep = prm->keep;
    p.maxiter = prm->maxiter;
    p.tol_resid = prm->tol_resid;
    p.switch_resid = prm->switch_resid;
    p.use_graph = prm->use_graph != 0;
    cg::BatchResult r;
    cg::batch_solve(b->bs, p, r);
    const int P = b->bs.np;
    for (size_t i = 0; i < size_t(P) * p.nev; ++i) {
      eig[i] = r.eig[i];
      if (resid) resid[i] = r.resid[i];
    }
    if (nconv)
      for (int i = 0; i < P; ++i) nconv[i] = r.nconv[i];
    if (stats) {
      stats->iterations_fp32 = r.iterations32;
      stats->iterations_fp64 = r.iterations64;
      stats->graph_launches = r.graph_launches;
      stats->graph_kernels = r.graph_kernels;
      stats->launches = r.launches;
      stats->seconds = r.seconds;
      stats->build_seconds = b->bs.build_seconds;
      stats->spmm_warps = b->bs.H.tuning.warps;
      stats->spmm_ctas_per_sm = b->bs.H.tuning.ctas_per_sm;
      stats->spmm_tune_seconds = b->bs.tune_seconds;
    }
  });
}

cg_status cg_jt_expectations(const cg_basis* b, const double* vecs, int32_t nstates, double* jj, double* tt) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(vecs);
    CG_NOT_NULL(jj);
    CG_NOT_NULL(tt);
    same_device(b->b.device);
    cg::jt_expectations(b->sys, b->b, vecs, nstates, jj, tt);
  });
}

int32_t cg_jj_spin(double jj, int32_t two_m) { return cg::jj_spin(jj, two_m); }

cg_status cg_xshlsf(const char* parent_xml, const char* parent_system, const char* daughter_xml,
                    const char* daughter_system, const char* out_path, int32_t full) {
  return guard([&] {
    CG_NOT_NULL(parent_xml);
    require_device();
    const std::string px = parent_xml, dx = daughter_xml ? daughter_xml : parent_xml;
    cg::xshlsf(px, parent_system ? parent_system : "", dx, daughter_system ? daughter_system : "",
               out_path ? out_path : "", full != 0);
    std::fflush(stdout);  // the tool's listing leaves the library with the call
  });
}

cg_status cg_transition_terms(const char* xml_path, const char* system_name, const char* op_name, int32_t kappa,
                              int32_t flags, int32_t* i, int32_t* f, double* v, int32_t cap, int32_t* count) {
  return guard([&] {
    CG_NOT_NULL(xml_path);
    CG_NOT_NULL(count);
    const cg::System sys = cg::load_system(xml_path, system_name ? system_name : "");
    const cg::XmlNode root = cg::parse_xml_file(xml_path);
    const cg::TransitionOp op = cg::read_transition_operator(root, op_name ? op_name : "",
                                                             (flags & CG_EMB_PHASE_INFINITY) != 0, nullptr, nullptr);
    const std::vector<cg::OneBodyTerm> t = cg::transition_terms(sys, op, kappa);
    *count = int32_t(t.size());
    if (cap == 0 && !i && !f && !v) return;
    CG_NOT_NULL(i);
    CG_NOT_NULL(f);
    CG_NOT_NULL(v);
    if (cap < int32_t(t.size())) throw cg::Error(CG_ERR_ARG, "cap below the number of terms");
    for (size_t k = 0; k < t.size(); ++k) {
      i[k] = t[k].i;
      f[k] = t[k].f;
      v[k] = t[k].v;
    }
  });
}

cg_status cg_onebody_amplitudes(const cg_basis* parent, const double* vp, int32_t np, const cg_basis* daughter,
                                const double* vd, int32_t nd, const int32_t* i, const int32_t* f, const double* v,
                                int32_t nterms, double* amp) {
  return guard([&] {
    CG_NOT_NULL(parent);
    CG_NOT_NULL(daughter);
    CG_NOT_NULL(vp);
    CG_NOT_NULL(vd);
    CG_NOT_NULL(amp);
    if (nterms < 0) throw cg::Error(CG_ERR_ARG, "negative term count");
    if (nterms) {
      CG_NOT_NULL(i);
      CG_NOT_NULL(f);
      CG_NOT_NULL(v);
    }
    same_device(parent->b.device);
    same_device(daughter->b.device);
    std::vector<cg::OneBodyTerm> t(nterms);
    for (int32_t k = 0; k < nterms; ++k) t[k] = {i[k], f[k], v[k]};
    cg::onebody_amplitudes(parent->sys, parent->b, vp, np, daughter->b, vd, nd, t, amp);
  });
}

cg_status cg_xshlemb(const char* parent_xml, const char* parent_system, const char* daughter_xml,
                     const char* daughter_system, const char* out_xml, int32_t flags, const char* op_name) {
  return guard([&] {
    CG_NOT_NULL(parent_xml);
    require_device();
    cg::XshlembOptions o;
    o.weisskopf = flags & CG_EMB_WEISSKOPF;
    o.units = flags & CG_EMB_UNITS;
    o.logft = flags & CG_EMB_LOGFT;
    o.phase_infinity = flags & CG_EMB_PHASE_INFINITY;
    o.op_name = op_name ? op_name : "";
    cg::xshlemb(parent_xml, parent_system ? parent_system : "", daughter_xml ? daughter_xml : "",
                daughter_system ? daughter_system : "", out_xml ? out_xml : "", o);
    std::fflush(stdout);  // the tool's listing leaves the library with the call
  });
}

cg_status cg_sf_amplitudes(const cg_basis* parent, const double* vp, int32_t np, const cg_basis* daughter,
                           const double* vd, int32_t nd, double* amp) {
  return guard([&] {
    CG_NOT_NULL(parent);
    CG_NOT_NULL(daughter);
    CG_NOT_NULL(vp);
    CG_NOT_NULL(vd);
    CG_NOT_NULL(amp);
    same_device(parent->b.device);
    same_device(daughter->b.device);
    cg::sf_amplitudes(parent->sys, parent->b, vp, np, daughter->b, vd, nd, amp);
  });
}

cg_status cg_xshljt(const char* xml_path, const char* system_name, const char* ee_path, int32_t nstates,
                    const char* xml_out, int32_t* n_added) {
  return guard([&] {
    CG_NOT_NULL(xml_path);
    CG_NOT_NULL(ee_path);
    const std::string sname = system_name ? system_name : "";
    cg::System sys = cg::load_system(xml_path, sname);
    require_device();
    cg::Basis b;
    cg::basis_build(sys, b);
    std::string file_attr = ee_path;
    auto states = cg::xshljt_states(sys, b, ee_path, nstates, file_attr, nullptr, nullptr);
    std::ifstream in(xml_path, std::ios::binary);
    if (!in) throw cg::Error(CG_ERR_IO, std::string("cannot open ") + xml_path);
    std::stringstream ss;
    ss << in.rdbuf();
    std::string text = cg::xml_add_states(ss.str(), sys.name, states);
    const char* dst = xml_out ? xml_out : xml_path;
    std::ofstream out(dst, std::ios::binary);
    if (!out) throw cg::Error(CG_ERR_IO, std::string("cannot write ") + dst);
    out << text;
    if (n_added) *n_added = int32_t(states.size());
  });
}

cg_status cg_gather_ceiling(uint64_t rows, int32_t share, double* gathers_per_second) {
  return guard([&] {
    CG_NOT_NULL(gathers_per_second);
    require_device();
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    *gathers_per_second = cg::gather_probe(dev, rows, share);
  });
}

cg_status cg_spmm_set_tuning(cg_hamiltonian* h, int32_t warps, int32_t ctas_per_sm) {
  return guard([&] {
    CG_NOT_NULL(h);
    if (warps != 4 && warps != 8 && warps != 16 && warps != 32) throw cg::Error(CG_ERR_ARG, "warps must be 4, 8, 16 or 32");
    if (ctas_per_sm < 1 || ctas_per_sm > 16) throw cg::Error(CG_ERR_ARG, "ctas_per_sm must be in 1..16");
    h->h.tuning.warps = warps;
    h->h.tuning.ctas_per_sm = ctas_per_sm;
    h->h.tuning.tuned = true;
  });
}

cg_status cg_spmm_get_tuning(const cg_hamiltonian* h, int32_t* warps, int32_t* ctas_per_sm, int32_t* tuned) {
  return guard([&] {
    CG_NOT_NULL(h);
    if (warps) *warps = h->h.tuning.warps;
    if (ctas_per_sm) *ctas_per_sm = h->h.tuning.ctas_per_sm;
    if (tuned) *tuned = h->h.tuning.tuned;
  });
}

cg_status cg_spmm_set_format(cg_hamiltonian* h, int32_t format) {
  return guard([&] {
    CG_NOT_NULL(h);
    if (format != CG_FORMAT_ROWS && format != CG_FORMAT_TILED) throw cg::Error(CG_ERR_ARG, "unknown SpMM format");
    if (format == CG_FORMAT_TILED && !h->h.tiled && !h->h.virt && h->h.precision == CG_PREC_FP32 &&
        !h->h.blocks.empty()) {
      CG_CUDA(cudaSetDevice(h->h.device));
      cg::tiled_build(h->h, h->h.blocks);  // built on request
    }
    if (format == CG_FORMAT_TILED && !h->h.tiled)
      throw cg::Error(CG_ERR_UNSUPPORTED,
                      "no block-tiled copy (needs an FP32 matrix built from a basis, blocks <= 1536 rows)");
    h->h.use_tiled = format == CG_FORMAT_TILED;
  });
}

cg_status cg_spmm_set_tiled_shape(cg_hamiltonian* h, int32_t slices_per_warp, int32_t stages) {
  return guard([&] {
    CG_NOT_NULL(h);
    cg::TiledOp* t = h->h.tiled.get();
    if (!t) throw cg::Error(CG_ERR_UNSUPPORTED, "no block-tiled copy");
    if (slices_per_warp < 1 || slices_per_warp > 4) throw cg::Error(CG_ERR_ARG, "slices per warp must be 1..4");
    const int warps = (t->smax + slices_per_warp - 1) / slices_per_warp;
    if (warps > 31) throw cg::Error(CG_ERR_ARG, "more than 31 consumer warps; take more slices per warp");
    if (stages < 2 || stages > 7 || cg::tiled_smem(*t, stages) > 227 * 1024)
      throw cg::Error(CG_ERR_ARG, "ring slots out of range (2..7 within 227 KB of shared memory)");
    t->rps = slices_per_warp;
    t->warps = warps;
    t->stages = stages;
  });
}

cg_status cg_spmm_get_format(const cg_hamiltonian* h, cg_spmm_format_info* info) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(info);
    *info = cg_spmm_format_info{};
    const cg::TiledOp* t = h->h.tiled.get();
    info->format = t && h->h.use_tiled ? CG_FORMAT_TILED : CG_FORMAT_ROWS;
    info->tiled_available = t != nullptr;
    if (t) {
      info->warps = t->warps;
      info->stages = t->stages;
      info->slices_per_warp = t->rps;
      info->entries = t->entries;
      info->units = t->nitems;
      info->meta_bytes = t->items.bytes() + t->rcopy.bytes() + t->iden.bytes();
      info->device_bytes = t->bytes();
      info->ident_tiles = t->ident_tiles;
      info->ident_entries = t->ident_nnz;
    }
  });
}

// -------------------------------------------------------------- Davidson
void cg_davidson_defaults(cg_davidson_params* prm, int32_t nstates) {
  if (!prm) return;
  std::memset(prm, 0, sizeof(*prm));
  prm->nstates = nstates;
  prm->block = nstates;
  prm->lim = nstates + 20;
  prm->maxiter = 0;
  prm->crite = 1e-15;
  prm->critc = 1e-12;
  prm->critr = 1e-8;
  prm->ortho = 1e-9;
  prm->tol_resid = 0.0;
  prm->switch_resid = 1e-3;
  prm->precision = CG_PREC_FP64;
  prm->verbose = 0;
  prm->ortho_block = 0;
  prm->algorithm = -1;
  prm->keep = 0;
  prm->precond = 1;
  prm->refine_lim = 0;
  prm->refine_keep = 0;
  prm->ortho_pip = 1;
  prm->refine_block = 0;
  prm->refine_fp32_corrections = 1;
}

cg_status cg_davidson(const cg_hamiltonian* h, const cg_davidson_params* prm, const double* init, int32_t n_init,
                      double* eig, double* de, double* resid, double* vecs, cg_davidson_stats* stats) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(prm);
    CG_NOT_NULL(eig);
    same_device(h->h.device);
    int nume = prm->nstates;
    if (nume < 1 || nume > 16) throw cg::Error(CG_ERR_ARG, "nstates must be in 1..16");
    if (uint64_t(nume) > h->h.n) throw cg::Error(CG_ERR_ARG, "nstates exceeds the dimension");
    if (prm->block < 1 || prm->block > nume) throw cg::Error(CG_ERR_ARG, "block must be in 1..nstates");
    if (prm->lim <= nume || prm->lim > 128) throw cg::Error(CG_ERR_ARG, "lim must be in nstates+1..128");
    if (n_init < 0 || (n_init > 0 && !init)) throw cg::Error(CG_ERR_ARG, "bad initial vectors");
    // a restart forms the kept Ritz vectors in place, at most 32 columns a pass
    if (prm->keep < 0 || prm->keep > 64) throw cg::Error(CG_ERR_ARG, "keep must be in 0..64");
    if (prm->refine_keep < 0 || prm->refine_keep > 64) throw cg::Error(CG_ERR_ARG, "refine_keep must be in 0..64");
    if (prm->precision != CG_PREC_FP64 && prm->precision != CG_PREC_FP32)
      throw cg::Error(CG_ERR_ARG, "precision must be CG_PREC_FP64 or CG_PREC_FP32");
    if (prm->precision != h->h.precision && !h->h.virt)
      throw cg::Error(CG_ERR_ARG, "Davidson precision must match the stored Hamiltonian precision");
    const double final_tol = prm->tol_resid > 0 ? prm->tol_resid : prm->critr;
    cg::DavConfig c;
    c.nume = nume;
    c.block = prm->block;
    c.lim = std::min<int64_t>(prm->lim, int64_t(h->h.n));
    if (c.lim <= nume) c.lim = nume;
    c.maxiter = prm->maxiter > 0 ? prm->maxiter : std::max(40 * nume, 200);
    c.crite = prm->crite;
    c.critc = prm->critc;
    c.critr = final_tol;
    c.ortho = prm->ortho;
    c.verbose = prm->verbose;
    // -1 (auto): the reference control flow for FP64, the residual-driven one for FP32
    const int algo = prm->algorithm < 0 ? (prm->precision == CG_PREC_FP32 ? 1 : 0) : prm->algorithm;
    if (algo != 0 && algo != 1) throw cg::Error(CG_ERR_ARG, "algorithm must be -1, 0 or 1");
    c.seq_ortho = !prm->ortho_block && algo == 0;
    c.modern = algo == 1;
    c.pip = algo == 1 && prm->ortho_pip != 0;
    c.keep = prm->keep;
    c.precond = prm->precond;
    cg::DavidsonRequest rq;
    rq.nume = nume;
    rq.init = init;
    rq.ninit = n_init;
    rq.vecs_out = vecs;
    if (prm->precision == CG_PREC_FP64) {
      c.spmm_prec = CG_PREC_FP64;
      rq.phase1 = c;
    } else {
      cg::DavConfig c1 = c;
      c1.spmm_prec = CG_PREC_FP32;
      c1.critr = std::max(prm->switch_resid, final_tol);
      c1.seq_ortho = false;  // FP32 vectors cannot reach the FP64 overlap threshold one vector at a time
      rq.phase1 = c1;
      cg::DavConfig c2 = c;
      c2.spmm_prec = CG_PREC_REFINE;
      if (prm->refine_lim > 0) {
        if (prm->refine_lim <= nume || prm->refine_lim > 128)
          throw cg::Error(CG_ERR_ARG, "refine_lim must be in nstates+1..128");
        c2.lim = prm->refine_lim;
      }
      if (prm->refine_keep > 0) c2.keep = prm->refine_keep;
      if (prm->refine_block > 0) {
        if (prm->refine_block > 16) throw cg::Error(CG_ERR_ARG, "refine_block must be in 1..16");
        c2.block = prm->refine_block;
      }
      c2.fp32_corr = prm->refine_fp32_corrections != 0;
      if (c2.keep + c2.block > c2.lim) c2.keep = std::max(nume, c2.lim - c2.block);

      rq.phase2 = c2;
      rq.refine = true;
    }
    if (prm->precision == CG_PREC_FP32 && !h->h.tuning.tuned && !h->h.virt)
      cg::spmm_autotune(const_cast<cg_hamiltonian*>(h)->h, std::min(prm->block, 16), 3);
    cg::DavResult r = cg::davidson_solve(h->h, rq);
    const cg::DavOutcome& f = r.final_;
    for (int i = 0; i < nume; ++i) {
      eig[i] = f.eig[i];
      if (de) de[i] = f.de[i];
      if (resid) resid[i] = f.resid[i];
    }
    if (stats) {
      stats->iterations = r.phase1.iterations + (r.refined ? r.phase2.iterations : 0);
      stats->refine_iterations = r.refined ? r.phase2.iterations : 0;
      stats->matvecs = r.phase1.matvecs + (r.refined ? r.phase2.matvecs : 0);
      stats->restarts = r.phase1.restarts + (r.refined ? r.phase2.restarts : 0);
      int conv = 0;
      for (int i = 0; i < nume; ++i) conv += f.resid[i] <= final_tol;
      stats->converged = conv;
      stats->ierr = f.ierr;
      stats->seconds = r.seconds;
      stats->spmm_seconds = r.phase1.spmm_seconds + (r.refined ? r.phase2.spmm_seconds : 0);
    }
  });
}

// ------------------------------------------------------------- file I/O
cg_status cg_occupations(const cg_basis* b, const double* vecs, int32_t nst, double* occ) {
  return guard([&] {
    CG_NOT_NULL(b);
    CG_NOT_NULL(occ);
    if (nst < 0) throw cg::Error(CG_ERR_ARG, "negative state count");
    if (nst) CG_NOT_NULL(vecs);
    same_device(b->b.device);
    cg::occupations(b->b, vecs, nst, occ);
  });
}

cg_status cg_xshlao(const char* xml_path, const char* system_name, const char* out_xml) {
  return guard([&] {
    CG_NOT_NULL(xml_path);
    require_device();
    cg::xshlao(xml_path, system_name ? system_name : "", out_xml ? out_xml : "");
    std::fflush(stdout);  // the tool's listing leaves the library with the call
  });
}

cg_status cg_xlevels(const char* const* files, int32_t nfiles, const char* out_xml) {
  return guard([&] {
    if (nfiles < 0) throw cg::Error(CG_ERR_ARG, "negative file count");
    if (nfiles) CG_NOT_NULL(files);
    std::vector<std::string> f;
    for (int32_t i = 0; i < nfiles; ++i) {
      CG_NOT_NULL(files[i]);
      f.emplace_back(files[i]);
    }
    std::fflush(stdout);
    const std::string out = cg::xlevels(f, out_xml ? out_xml : "");
    std::fwrite(out.data(), 1, out.size(), stdout);
    std::fflush(stdout);
  });
}

cg_status cg_dense_eigensolve(const cg_hamiltonian* h, double* eig, double* vecs) {
  return guard([&] {
    CG_NOT_NULL(h);
    CG_NOT_NULL(eig);
    if (h->h.virt) throw cg::Error(CG_ERR_UNSUPPORTED, "exact diagonalization needs a stored matrix");
    const uint64_t n = h->h.n;
    if (n > 8192) throw cg::Error(CG_ERR_ARG, "exact diagonalization takes at most 8192 states");
    if (n == 0) return;
    same_device(h->h.device);
    std::vector<uint64_t> rp(n + 1);
    cg::hamiltonian_upper_rows(h->h, 0, n, rp.data(), nullptr, nullptr);
    std::vector<uint32_t> c(rp[n]);
    std::vector<double> v(rp[n]);
    cg::hamiltonian_upper_rows(h->h, 0, n, rp.data(), c.data(), v.data());
    std::vector<double> a(n * n, 0.0), w, z;
    for (uint64_t r = 0; r < n; ++r)
      for (uint64_t k = rp[r]; k < rp[r + 1]; ++k) {
        a[r * n + c[k]] = v[k];
        a[uint64_t(c[k]) * n + r] = v[k];
      }
    cg::sym_eig(int(n), a, w, z);
    for (uint64_t k = 0; k < n; ++k) eig[k] = w[k];
    if (vecs)
      for (uint64_t k = 0; k < n; ++k)
        for (uint64_t i = 0; i < n; ++i) vecs[k * n + i] = z[i * n + k];
  });
}

cg_status cg_write_ee(const char* path, int32_t nstates, uint64_t n, const double* eig, const double* de,
                      const double* resid, const double* vecs) {
  return guard([&] {
    CG_NOT_NULL(path);
    CG_NOT_NULL(eig);
    CG_NOT_NULL(de);
    CG_NOT_NULL(resid);
    CG_NOT_NULL(vecs);
    std::ofstream f(path, std::ios::binary);
    if (!f) throw cg::Error(CG_ERR_IO, std::string("cannot write ") + path);
    uint32_t cnt = uint32_t(nstates);
    f.write(reinterpret_cast<const char*>(&cnt), 4);
    for (int i = 0; i < nstates; ++i) {
      f.write(reinterpret_cast<const char*>(eig + i), 8);
      f.write(reinterpret_cast<const char*>(de + i), 8);
      f.write(reinterpret_cast<const char*>(resid + i), 8);
      f.write(reinterpret_cast<const char*>(&n), 8);
      f.write(reinterpret_cast<const char*>(vecs + uint64_t(i) * n), 8 * n);
    }
    if (!f) throw cg::Error(CG_ERR_IO, std::string("write failed: ") + path);
  });
}

}  // extern "C"
