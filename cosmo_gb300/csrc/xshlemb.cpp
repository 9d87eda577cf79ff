// XSHLEMB: electromagnetic and beta transition rates between the states of a
// parent and a daughter system (xmlshell/XSHLEMB.cpp:116-372).
//
// The operator is the <operator> child of the parent XML's root
// (include/xsm/xmlemb.cxx:121-221): name E<K> / M<K> / GT+ / GT- / F, J = K,
// effective charges en, ep for E; mu_n, mu_p, gl_n, gl_p for M (the free
// values when absent, then added to the node as the reference's
// InquireAttribute does).  Its m-scheme terms for the projection
// kappa = (Jz_daughter - Jz_parent) / 2 of the systems (em.cpp) act on every
// parent state on the GPU (sf.cu, onebody_amplitudes), giving
// x = <D| O |P>.  For every parent state p and daughter state q with a
// nonzero <J_D Jz_D, K Jz_P - Jz_D | J_P Jz_P> = c, B = (x / c)^2 is written as
// <transition name="B(op)" final E [units] B [weisskopf] [Bu] [logft]/>
// appended to the parent state; a diagonal element (same energy from the .EE
// file, J, T and Tz, K < 3) also gets <moment name m [oscl]/> as its first
// child, m = x / c <J_D J_D, K 0 | J_P J_P> sqrt(4 pi / (2K + 1)) K.
// Numbers are written in the default C++ stream format (6 significant
// digits), as the reference's addAttribute does.
#include <cmath>
#include <iostream>
#include <fstream>
#include <sstream>

#include "cosmo_gb300.h"
#include "device.h"
#include "em.h"
#include "model.h"
#include "xshljt.h"

namespace cg {

namespace {

constexpr double kPi = 3.141592653589793238462643;

const XmlNode* find_system_node(const XmlNode& root, const std::string& name) {
  for (int i = 0; i < root.count("system"); ++i) {
    const XmlNode* c = root.child("system", i);
    if (name.empty() || (c->attr("name") && *c->attr("name") == name)) return c;
  }
  return nullptr;
}

// attribute, else child element text (getXMLData)
const std::string* xml_data(const XmlNode& n, const std::string& key) {
  if (const std::string* a = n.attr(key)) return a;
  if (const XmlNode* c = n.child(key)) return &c->text;
  return nullptr;
}

}  // namespace

TransitionOp read_transition_operator(const XmlNode& root, const std::string& op_name, bool phase_infinity, int* index,
                                      std::vector<std::pair<std::string, std::string>>* added) {
  const int nops = root.count("operator");
  if (nops == 0) throw Error(CG_ERR_ARG, "no <operator> node in the XML");
  int opi = 0;
  if (!op_name.empty()) {
    opi = -1;
    for (int i = 0; i < nops; ++i)
      if (root.child("operator", i)->attr("name") && *root.child("operator", i)->attr("name") == op_name) opi = i;
    if (opi < 0) throw Error(CG_ERR_ARG, "no <operator name=\"" + op_name + "\">");
  }
  const XmlNode& on = *root.child("operator", opi);
  TransitionOp op;
  op.name = on.attr("name") ? *on.attr("name") : std::string();
  if (op.name.empty()) throw Error(CG_ERR_PARSE, "<operator> without a name");
  const std::string* kj = xml_data(on, "J");
  op.K = kj ? std::atoi(kj->c_str()) : 2;
  op.origin_positive = !phase_infinity;
  if (on.child("radial"))
    throw Error(CG_ERR_UNSUPPORTED, "radial overlaps from a file (<radial>): only oscillator radial functions");
  const char type = op.name[0];
  if (type == 'E') {
    const std::string *en = xml_data(on, "en"), *ep = xml_data(on, "ep");
    if (!en || !ep) throw Error(CG_ERR_ARG, "an E operator needs the effective charges en and ep");
    op.en = std::atof(en->c_str());
    op.ep = std::atof(ep->c_str());
  } else if (type == 'M') {
    struct {
      const char* key;
      double* v;
    } ms[4] = {{"mu_n", &op.mu_n}, {"mu_p", &op.mu_p}, {"gl_n", &op.gl_n}, {"gl_p", &op.gl_p}};
    for (auto& m : ms) {
      if (const std::string* t = xml_data(on, m.key)) *m.v = std::atof(t->c_str());
      else if (added) added->emplace_back(m.key, num_text(*m.v));
    }
  } else if (type == 'G') {
    if (op.name != "GT+" && op.name != "GT-") throw Error(CG_ERR_ARG, "beta operator " + op.name + ": GT+ or GT-");
    if (op.K != 1) throw Error(CG_ERR_ARG, "the Gamow-Teller operator has J = 1");
  } else if (type == 'F') {
    if (op.K != 0) throw Error(CG_ERR_ARG, "the Fermi operator is a scalar (J = 0)");
  } else {
    throw Error(CG_ERR_ARG, "operator " + op.name + ": not E, M, GT+, GT- or F");
  }
  if (index) *index = opi;
  return op;
}

void xshlemb(const std::string& pxml, const std::string& psys_name, const std::string& dxml_in,
             const std::string& dsys_name, const std::string& out_xml, const XshlembOptions& opt) {
  const std::string dxml = dxml_in.empty() ? pxml : dxml_in;
  const System ps = load_system(pxml, psys_name);
  const System ds = load_system(dxml, dsys_name);
  if (ps.sps.size() != ds.sps.size() || ps.n_neutron_states != ds.n_neutron_states)
    throw Error(CG_ERR_ARG, "parent and daughter systems have different valence spaces");
  // the operator node
  const XmlNode root = parse_xml_file(pxml);
  int opi = 0;
  std::vector<std::pair<std::string, std::string>> added;
  const TransitionOp op = read_transition_operator(root, opt.op_name, opt.phase_infinity, &opi, &added);
  const char type = op.name[0];
  if ((ds.twom - ps.twom) & 1) throw Error(CG_ERR_ARG, "parent and daughter Jz differ by a half-integer");
  const int kappa = (ds.twom - ps.twom) / 2;
  const std::vector<OneBodyTerm> terms = transition_terms(ps, op, kappa);

  // mass number for the unit conversions
  int A = 1;
  {
    const XmlNode* sn = find_system_node(root, ps.name);
    const std::string* a = sn ? xml_data(*sn, "A") : nullptr;
    if (a) A = std::atoi(a->c_str());
    else if (opt.weisskopf || opt.units)
      std::cerr << "Nuclear mass number A is not defined, units will not work\n";
  }

  // states, vectors, amplitudes
  const std::vector<StateRecord> pst = read_states(pxml, ps.name), dst = read_states(dxml, ds.name);
  Basis pb, db;
  basis_build(ps, pb);
  basis_build(ds, db);
  const int np = int(pst.size()), nd = int(dst.size());
  std::vector<double> pv, dv, pE(np), dE(nd);
  for (int p = 0; p < np; ++p) {
    const auto v = read_vector(pst[p].file, dir_of(pxml), pst[p].id, pb.n, &pE[p]);
    pv.insert(pv.end(), v.begin(), v.end());
  }
  for (int q = 0; q < nd; ++q) {
    const auto v = read_vector(dst[q].file, dir_of(dxml), dst[q].id, db.n, &dE[q]);
    dv.insert(dv.end(), v.begin(), v.end());
  }
  std::vector<double> amp(size_t(nd) * np, 0.0), part;
  for (int q0 = 0; q0 < nd; q0 += 16) {
    const int m = std::min(16, nd - q0);
    part.assign(size_t(m) * np, 0.0);
    onebody_amplitudes(ps, pb, pv.data(), np, db, dv.data() + size_t(q0) * db.n, m, terms, part.data());
    for (size_t i = 0; i < part.size(); ++i) amp[size_t(q0) * np + i] = part[i];
  }

  // transitions and moments
  const std::string bname = "B(" + op.name + ")";
  std::vector<std::vector<std::string>> front(np), back(np);
  for (int p = 0; p < np; ++p) {
    const StateRecord& P = pst[p];
    double bsum = 0.0;
    std::cout << "\n";
    for (int q = 0; q < nd; ++q) {
      const StateRecord& D = dst[q];
      const int jz = P.twoJz - D.twoJz;
      const double c = clebsch_gordan(D.twoJ, D.twoJz, 2 * op.K, jz, P.twoJ, P.twoJz);
      if (std::fabs(c) < 1e-10) continue;
      const double x = amp[size_t(q) * np + p];
      const double B = (x / c) * (x / c);
      const double t3 = three_j(D.twoJ, -D.twoJz, 2 * op.K, -jz, P.twoJ, P.twoJz) *
                        (((D.twoJ - D.twoJz) / 2 & 1) ? -1.0 : 1.0);
      bsum += B;
      std::cout << D.twoJ << " " << D.twoJz << " " << 2 * op.K << " " << jz << " " << P.twoJ << " " << P.twoJz
                << "  M=" << x / t3 << " B=" << B << "  sum=" << bsum;
      double w = -1.0, bu = -1.0;
      if (opt.weisskopf) {
        w = weisskopf_units(type, op.K, A, B);
        if (w > -1) std::cout << " W=" << w;
      }
      if (opt.units) {
        bu = standard_units(type, op.K, A, B);
        if (bu > -1) std::cout << " Bu=" << bu;
      }
      std::cout << "\n";
      std::string tr = "<transition name=\"" + bname + "\" final=\"" + D.name + "\" E=\"" + D.e_text + "\"";
      if (type == 'G') tr += " units=\"ga^2/(4pi)\"";
      tr += " B=\"" + num_text(B) + "\"";
      if (opt.weisskopf && w > -1) tr += " weisskopf=\"" + num_text(w) + "\"";
      if (opt.units && bu > -1) tr += " Bu=\"" + num_text(bu) + "\"";
      if (opt.logft) tr += " logft=\"" + num_text(std::log(6145.0 / 1.27 / 1.27 / B) / std::log(10.0)) + "\"";
      back[p].push_back(tr + "/>");
      if (std::fabs(pE[p] - dE[q]) < 1e-5 && P.twoJ == D.twoJ && P.twoT == D.twoT && op.K < 3 &&
          P.twoTz == D.twoTz) {
        const double mm = x / c * clebsch_gordan(D.twoJ, D.twoJ, 2 * op.K, 0, P.twoJ, P.twoJ) *
                          std::sqrt(4.0 * kPi / (2.0 * op.K + 1)) * op.K;
        std::string mo = "<moment name=\"" + op.name + "\" m=\"" + num_text(mm) + "\"";
        if (opt.units) mo += " oscl=\"" + num_text(std::sqrt(oscillator_b2(A))) + "\"";
        front[p].insert(front[p].begin(), mo + "/>");
      }
    }
  }

  std::ifstream in(pxml, std::ios::binary);
  std::stringstream ss;
  ss << in.rdbuf();
  std::string text = ss.str();
  if (!added.empty()) text = xml_append_attrs(text, "operator", opi, added);
  text = xml_state_children(text, ps.name, front, back);
  const std::string dst_path = out_xml.empty() ? pxml : out_xml;
  std::ofstream of(dst_path, std::ios::binary);
  if (!of) throw Error(CG_ERR_IO, "cannot write " + dst_path);
  of << text;
}

// XSHLAO (xmlshell/XSHLAO.cpp:22-101): occupation numbers of every orbital,
// neutrons and protons apart, for every <state> of the system, written as
// <occupation name N Z/> children of the states (orbitals in the document
// order of the valence space, as the reference walks them).
void xshlao(const std::string& xml, const std::string& system_name, const std::string& out_xml) {
  const System sys = load_system(xml, system_name);
  const XmlNode root = parse_xml_file(xml);
  const XmlNode* vs = root.child("valencespace");
  if (!vs) throw Error(CG_ERR_PARSE, "no <valencespace>");
  const std::vector<StateRecord> st = read_states(xml, sys.name);
  Basis b;
  basis_build(sys, b);
  const int nst = int(st.size()), ns = int(sys.sps.size());
  std::vector<double> v;
  for (const StateRecord& r : st) {
    const auto x = read_vector(r.file, dir_of(xml), r.id, b.n, nullptr);
    v.insert(v.end(), x.begin(), x.end());
  }
  std::vector<double> occ(size_t(nst) * ns);
  occupations(b, v.data(), nst, occ.data());
  std::vector<std::vector<std::string>> front(nst), back(nst);
  for (int k = 0; k < nst; ++k) {
    std::cout << st[k].name << " E=" << st[k].e_text << "\n";
    for (int o = 0; o < vs->count("orbital"); ++o) {
      const XmlNode* orb = vs->child("orbital", o);
      const std::string name = orb->attr("name") ? *orb->attr("name") : std::string();
      const int level = orb->attr("index") ? std::atoi(orb->attr("index")->c_str()) - 1 : o;
      double occN = 0.0, occZ = 0.0;
      for (int i = 0; i < ns; ++i)
        if (sys.sps[i].level == level) (sys.sps[i].tz2 == 1 ? occN : occZ) += occ[size_t(k) * ns + i];
      back[k].push_back("<occupation name=\"" + name + "\" N=\"" + num_text(occN) + "\" Z=\"" + num_text(occZ) + "\"/>");
      std::cout << "  " << name << " N=" << occN << " Z=" << occZ << "\n";
    }
  }
  std::ifstream in(xml, std::ios::binary);
  std::stringstream ss;
  ss << in.rdbuf();
  const std::string text = xml_state_children(ss.str(), sys.name, front, back);
  const std::string dst = out_xml.empty() ? xml : out_xml;
  std::ofstream of(dst, std::ios::binary);
  if (!of) throw Error(CG_ERR_IO, "cannot write " + dst);
  of << text;
}

}  // namespace cg
