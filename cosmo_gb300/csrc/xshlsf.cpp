// XSHLSF: spectroscopic factors of one-particle removal between the states of
// a parent and a daughter system (xmlshell/XSHLSF.cpp:40-222).
//
// Both systems come from XML files with <state> children (as XSHLJT writes
// them: J, T, P, E, name, Ex, and a <wavefunction Jz Tz file id> child naming
// the .EE eigenvector file and index, include/xsm/xState.cxx:23-46).  For
// every parent state p and daughter state q with one particle less, and every
// s.p. state s with m_s = Jz(p) - Jz(q), tz_s = Tz(p) - Tz(q) and the parity
// change, the amplitude A = <q| a_s |p> / <J_q Jz_q, j_s m_s | J_p Jz_p> (the
// overlap on the GPU, sf.cu) and SF = A^2; SFs are summed per orbital l.  With
// equal particle numbers the overlap <q|p> of states with the same J, T, Jz,
// Tz and parity is printed instead.  The output file has the reference's
// layout: a header, then "parent Ex daughter Ex L SF" per l, or with `full`
// "parent Ex daughter Ex L 2j A SF" per s.p. state.
#include <cmath>
#include <cstdio>
#include <fstream>
#include <iostream>
#include <sstream>

#include "cosmo_gb300.h"
#include "device.h"
#include "model.h"
#include "xshljt.h"

namespace cg {

// the <state> children of the system node (ReadXMLState, include/xsm/xState.cxx:38-46)
std::vector<StateRecord> read_states(const std::string& xml_path, const std::string& system_name) {
  XmlNode root = parse_xml_file(xml_path);
  const XmlNode* sn = nullptr;
  const int ns = root.count("system");
  for (int i = 0; i < ns; ++i) {
    const XmlNode* c = root.child("system", i);
    if (system_name.empty() || (c->attr("name") && *c->attr("name") == system_name)) {
      sn = c;
      break;
    }
  }
  if (!sn) throw Error(CG_ERR_ARG, "no system " + system_name + " in " + xml_path);
  std::vector<StateRecord> out;
  for (int i = 0; i < sn->count("state"); ++i) {
    const XmlNode* st = sn->child("state", i);
    const XmlNode* wf = st->child("wavefunction");
    if (!wf || !wf->attr("file") || !wf->attr("id")) throw Error(CG_ERR_PARSE, "a <state> without its wave function");
    StateRecord s;
    s.name = st->attr("name") ? *st->attr("name") : std::string();
    s.ex = st->attr("Ex") ? *st->attr("Ex") : std::string();
    s.e_text = st->attr("E") ? *st->attr("E") : std::string();
    if (!st->attr("J")) throw Error(CG_ERR_PARSE, "a <state> without J");
    s.twoJ = parse_spin2(*st->attr("J"));
    s.twoT = st->attr("T") ? parse_spin2(*st->attr("T")) : -1;
    s.parity = st->attr("P") && (*st->attr("P"))[0] == '-' ? 1 : 0;
    s.E = st->attr("E") ? std::atof(st->attr("E")->c_str()) : 0.0;
    s.twoJz = wf->attr("Jz") ? parse_spin2(*wf->attr("Jz")) : 0;
    s.twoTz = wf->attr("Tz") ? parse_spin2(*wf->attr("Tz")) : 0;
    s.file = *wf->attr("file");
    s.id = std::atoi(wf->attr("id")->c_str());
    out.push_back(s);
  }
  if (out.empty()) throw Error(CG_ERR_ARG, "no states in the system " + system_name + " of " + xml_path);
  return out;
}

// vector `id` of an .EE file and its energy (SM::EnergyStateRead), looked up
// as given, then beside the XML file
std::vector<double> read_vector(const std::string& file, const std::string& xml_dir, int id, uint64_t n,
                                double* energy) {
  std::ifstream f(file, std::ios::binary);
  if (!f && !xml_dir.empty()) f.open(xml_dir + "/" + file, std::ios::binary);
  if (!f) throw Error(CG_ERR_IO, "cannot open " + file);
  uint32_t count = 0;
  f.read(reinterpret_cast<char*>(&count), 4);
  if (!f || id < 0 || uint32_t(id) >= count) throw Error(CG_ERR_IO, "no vector " + std::to_string(id) + " in " + file);
  std::vector<double> v(n);
  for (int k = 0; k <= id; ++k) {
    double e[3];
    uint64_t m = 0;
    f.read(reinterpret_cast<char*>(e), 24);
    f.read(reinterpret_cast<char*>(&m), 8);
    if (!f || m != n) throw Error(CG_ERR_IO, ".EE vector dimension does not match the basis: " + file);
    if (energy) *energy = e[0];
    if (k < id) f.seekg(std::streamoff(8 * m), std::ios::cur);
    else f.read(reinterpret_cast<char*>(v.data()), std::streamsize(8 * n));
  }
  if (!f) throw Error(CG_ERR_IO, "short .EE file " + file);
  return v;
}

std::string dir_of(const std::string& p) {
  const size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string() : p.substr(0, s);
}

void xshlsf(const std::string& pxml, const std::string& psys_name, const std::string& dxml,
            const std::string& dsys_name, const std::string& out_path, bool full) {
  const System ps = load_system(pxml, psys_name);
  const System ds = load_system(dxml, dsys_name);
  if (ps.sps.size() != ds.sps.size() || ps.n_neutron_states != ds.n_neutron_states)
    throw Error(CG_ERR_ARG, "parent and daughter systems have different valence spaces");
  const std::vector<StateRecord> pst = read_states(pxml, ps.name), dst = read_states(dxml, ds.name);
  const int NP = ps.nv + ps.zv, ND = ds.nv + ds.zv;
  if (NP != ND && NP - ND != 1)
    throw Error(CG_ERR_ARG, "the number of particles in the final system must be less by one than in the initial");
  Basis pb, db;
  basis_build(ps, pb);
  basis_build(ds, db);
  std::vector<double> pv, dv;
  for (const StateRecord& s : pst) {
    const auto v = read_vector(s.file, dir_of(pxml), s.id, pb.n, nullptr);
    pv.insert(pv.end(), v.begin(), v.end());
  }
  for (const StateRecord& s : dst) {
    const auto v = read_vector(s.file, dir_of(dxml), s.id, db.n, nullptr);
    dv.insert(dv.end(), v.begin(), v.end());
  }
  const int np = int(pst.size()), nd = int(dst.size()), ns = int(ps.sps.size());
  std::vector<double> amp;
  if (NP - ND == 1) {
    amp.assign(size_t(nd) * np * ns, 0.0);
    std::vector<double> part(size_t(std::min(nd, 16)) * np * ns);
    for (int q0 = 0; q0 < nd; q0 += 16) {
      const int m = std::min(16, nd - q0);
      sf_amplitudes(ps, pb, pv.data(), np, db, dv.data() + size_t(q0) * db.n, m, part.data());
      for (size_t i = 0; i < size_t(m) * np * ns; ++i) amp[size_t(q0) * np * ns + i] = part[i];
    }
  }
  std::ofstream of;
  if (!out_path.empty()) {
    of.open(out_path);
    if (!of) throw Error(CG_ERR_IO, "cannot write " + out_path);
    of << "#Spectroscopic factors for transition between " << ps.name << " and " << ds.name << "\n";
    of << "#File: " << pxml << " ";
    if (dxml != pxml) of << "Final(daugter) system file: " << dxml;
    of << "\n";
    of << (full ? "#parent Ex(p) daugther Ex(d) L J A SF=|A|^2 \n" : "#parent Ex(p) daugther Ex(d) L SF=|A|^2 \n");
  }
  for (int p = 0; p < np; ++p) {
    const StateRecord& P = pst[p];
    for (int q = 0; q < nd; ++q) {
      const StateRecord& D = dst[q];
      const int jz = P.twoJz - D.twoJz, tz = P.twoTz - D.twoTz, par = P.parity ^ D.parity;
      std::cout << "Parent: " << P.name << " Ex=" << P.ex << " E=" << P.E << "\n";
      std::cout << "Daughter: " << D.name << " Ex=" << D.ex << " E=" << D.E << "\n";
      if (NP == ND) {
        if (jz || tz || par || P.twoJ != D.twoJ || P.twoT != D.twoT) continue;
        double ov = 0.0;
        for (uint64_t i = 0; i < pb.n; ++i) ov += dv[size_t(q) * db.n + i] * pv[size_t(p) * pb.n + i];
        std::cout << "<x|y> " << ov << " |<x|y>|^2 = " << ov * ov << " \n";
        continue;
      }
      std::vector<double> lsf(20, 0.0);
      for (int s = 0; s < ns; ++s) {
        const SPState& sp = ps.sps[s];
        if (sp.m2 != jz || sp.tz2 != tz || (sp.parity ^ par)) continue;
        const double cgc = clebsch_gordan(D.twoJ, D.twoJz, sp.j2, jz, P.twoJ, P.twoJz);
        if (std::fabs(cgc) < 1e-10) continue;
        const double a = amp[(size_t(q) * np + p) * ns + s] / cgc;
        std::cout << "l=" << sp.l << " j=" << sp.j2 << "/2 C2S=" << a * a << " A=" << a << "\n";
        if (full && of) {
          of << P.name << "\t" << P.ex << "\t" << D.name << "\t" << D.ex << "\t" << sp.l << "\t" << spin_text(sp.j2) << "\t" << a
             << "\t " << a * a << "\n";
        }
        if (sp.l < int(lsf.size())) lsf[sp.l] += a * a;
      }
      std::cout << "\n";
      if (!full && of)
        for (int l = 0; l < int(lsf.size()); ++l)
          if (lsf[l] > 0) of << P.name << "\t" << P.ex << "\t" << D.name << "\t" << D.ex << "\t" << l << "\t" << lsf[l] << "\n";
    }
  }
}

}  // namespace cg
