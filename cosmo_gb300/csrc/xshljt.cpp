// XSHLJT on the GPU path: spin / isospin assignment of eigenpairs and the
// <state> database nodes of the system XML.
//
// Reference: xsm::XSHLJT (include/xsm/XSHLJT.cxx:38-142) reads the .EE file,
// computes <J-J+> and <T-T+> per state (PPMatrix::Sqr), converts them to 2J / 2T
// (SM::JJSpin, include/sm/QN.cxx:40-60), removes the lambda * J-J+ penalty from
// the energy (:114-117), and records each state with SM::AddState followed by
// SM::OrganizeStates (include/xsm/xState.cxx:113-236).  The XML text outside the
// system's <state> children is kept byte for byte; the <state> children are
// regenerated in energy order with the reference's attribute order
// (J P T E dE name Ex; wavefunction Jz Tz file id), names "J" P "(k)" counted
// per (J, P), Ex from the written energies, and numbers in the default C++
// stream format the reference's updateAttribute uses (6 significant digits).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <sstream>

#include "device.h"
#include "xshljt.h"

namespace cg {

namespace {

using Attrs = std::vector<std::pair<std::string, std::string>>;

struct StateNode {
  Attrs attrs;
  std::vector<Attrs> wfs;
  // the children in document order: an empty string stands for the next
  // <wavefunction> of wfs, anything else is another child element kept as
  // written (<transition>, <moment>, ... of other tools)
  std::vector<std::string> kids;
};

std::string num_str(double x) {
  std::ostringstream ss;
  ss << x;
  return ss.str();
}

const std::string* get(const Attrs& a, const std::string& k) {
  for (auto& kv : a)
    if (kv.first == k) return &kv.second;
  return nullptr;
}

// updateAttribute: an existing attribute is deleted and the new value appended
void update(Attrs& a, const std::string& k, const std::string& v) {
  a.erase(std::remove_if(a.begin(), a.end(), [&](const std::pair<std::string, std::string>& kv) { return kv.first == k; }),
          a.end());
  a.emplace_back(k, v);
}

bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }

// attributes of a start tag text "<tag a="1" b='2' ...>" beginning at `p`
Attrs parse_attrs(const std::string& s, size_t p, size_t end) {
  Attrs a;
  while (p < end && !is_space(s[p]) && s[p] != '>' && s[p] != '/') ++p;  // tag name
  while (p < end) {
    while (p < end && is_space(s[p])) ++p;
    if (p >= end || s[p] == '>' || s[p] == '/') break;
    size_t k0 = p;
    while (p < end && s[p] != '=' && !is_space(s[p])) ++p;
    std::string key = s.substr(k0, p - k0);
    while (p < end && (is_space(s[p]) || s[p] == '=')) ++p;
    if (p >= end) break;
    char q = s[p];
    if (q != '"' && q != '\'') throw Error(CG_ERR_PARSE, "xml: unquoted attribute " + key);
    size_t v0 = ++p;
    while (p < end && s[p] != q) ++p;
    a.emplace_back(key, s.substr(v0, p - v0));
    ++p;
  }
  return a;
}

// position of the next start tag "<name" (followed by space, '>' or '/') at or after p
size_t find_tag(const std::string& s, const std::string& name, size_t p, size_t end) {
  const std::string open = "<" + name;
  while (true) {
    size_t q = s.find(open, p);
    if (q == std::string::npos || q >= end) return std::string::npos;
    size_t r = q + open.size();
    if (r < s.size() && (is_space(s[r]) || s[r] == '>' || s[r] == '/')) return q;
    p = r;
  }
}

size_t tag_end(const std::string& s, size_t p) {  // index of the '>' closing the tag at p
  char q = 0;
  for (size_t i = p; i < s.size(); ++i) {
    if (q) {
      if (s[i] == q) q = 0;
    } else if (s[i] == '"' || s[i] == '\'') {
      q = s[i];
    } else if (s[i] == '>') {
      return i;
    }
  }
  throw Error(CG_ERR_PARSE, "xml: unterminated tag");
}

std::string attrs_text(const Attrs& a) {
  std::string t;
  for (auto& kv : a) t += " " + kv.first + "=\"" + kv.second + "\"";
  return t;
}

// The <state> children of a system body (attributes, wavefunctions and the
// other children as written), removed from the body.
std::vector<StateNode> take_states(std::string& body) {
  std::vector<StateNode> states;
  std::string kept;
  size_t q = 0;
  while (true) {
    size_t st = find_tag(body, "state", q, body.size());
    if (st == std::string::npos) {
      kept += body.substr(q);
      break;
    }
    size_t ls = st;
    while (ls > q && (body[ls - 1] == ' ' || body[ls - 1] == '\t')) --ls;
    if (ls > q && body[ls - 1] == '\n') --ls;
    kept += body.substr(q, ls - q);
    const size_t e = tag_end(body, st);
    StateNode sn;
    sn.attrs = parse_attrs(body, st + 1, e);
    size_t next = e + 1;
    if (body[e - 1] != '/') {
      size_t close = body.find("</state>", e);
      if (close == std::string::npos) throw Error(CG_ERR_PARSE, "xml: </state> missing");
      size_t w = e + 1;
      while (true) {
        const size_t c0 = body.find('<', w);
        if (c0 == std::string::npos || c0 >= close) break;
        const size_t ce = tag_end(body, c0);
        size_t n0 = c0 + 1;
        while (n0 < ce && !is_space(body[n0]) && body[n0] != '/' && body[n0] != '>') ++n0;
        const std::string name = body.substr(c0 + 1, n0 - c0 - 1);
        size_t end = ce + 1;  // past the child element
        if (body[ce - 1] != '/' && name[0] != '!' && name[0] != '?') {
          const size_t cl = body.find("</" + name + ">", ce);
          if (cl == std::string::npos || cl > close) throw Error(CG_ERR_PARSE, "xml: </" + name + "> missing");
          end = cl + name.size() + 3;
        }
        if (name == "wavefunction") {
          sn.wfs.push_back(parse_attrs(body, c0 + 1, ce));
          sn.kids.emplace_back();
        } else {
          sn.kids.push_back(body.substr(c0, end - c0));
        }
        w = end;
      }
      next = close + 8;
    }
    states.push_back(std::move(sn));
    q = next;
  }
  body = kept;
  return states;
}

}  // namespace

std::string spin_text(int twice) {
  char b[24];
  if (twice & 1) std::snprintf(b, sizeof b, "%i/2", twice);
  else std::snprintf(b, sizeof b, "%i", twice >> 1);
  return b;
}

std::string num_text(double x) { return num_str(x); }

namespace {

// [start, end) of the system element's start tag and the position of its
// end tag (npos for a self-closed system)
void find_system(const std::string& text, const std::string& system_name, size_t& start, size_t& stag_end,
                 size_t& close) {
  size_t p = 0;
  start = std::string::npos;
  while ((p = find_tag(text, "system", p, text.size())) != std::string::npos) {
    const size_t e = tag_end(text, p);
    Attrs a = parse_attrs(text, p + 1, e);
    const std::string* nm = get(a, "name");
    if (system_name.empty() || (nm && *nm == system_name)) {
      start = p;
      break;
    }
    p = e;
  }
  if (start == std::string::npos) throw Error(CG_ERR_PARSE, "xml: system " + system_name + " not found");
  stag_end = tag_end(text, start);
  close = text[stag_end - 1] == '/' ? std::string::npos : text.find("</system>", stag_end);
}

std::string line_indent(const std::string& text, size_t p) {
  const size_t ls = text.rfind('\n', p);
  const size_t b = ls == std::string::npos ? 0 : ls + 1;
  std::string in = text.substr(b, p - b);
  for (char& c : in)
    if (!is_space(c)) c = ' ';
  return in;
}

}  // namespace

std::string xml_state_children(const std::string& text, const std::string& system_name,
                               const std::vector<std::vector<std::string>>& front,
                               const std::vector<std::vector<std::string>>& back) {
  size_t sys, stag_end, close;
  find_system(text, system_name, sys, stag_end, close);
  if (close == std::string::npos) {
    if (!front.empty() || !back.empty()) throw Error(CG_ERR_PARSE, "xml: the system has no <state> children");
    return text;
  }
  std::string out = text.substr(0, stag_end + 1);
  size_t q = stag_end + 1;
  size_t k = 0;
  while (true) {
    const size_t st = find_tag(text, "state", q, close);
    if (st == std::string::npos) break;
    const size_t e = tag_end(text, st);
    const std::string in = line_indent(text, st) + "\t";
    std::string fr, bk;
    if (k < front.size())
      for (const std::string& c : front[k]) fr += "\n" + in + c;
    if (k < back.size())
      for (const std::string& c : back[k]) bk += "\n" + in + c;
    if (text[e - 1] == '/') {  // <state .../>
      out += text.substr(q, e - 1 - q);
      if (fr.empty() && bk.empty()) {
        out += "/>";
      } else {
        out += ">" + fr + bk + "\n" + line_indent(text, st) + "</state>";
      }
      q = e + 1;
    } else {
      const size_t end = text.find("</state>", e);
      if (end == std::string::npos || end > close) throw Error(CG_ERR_PARSE, "xml: </state> missing");
      size_t tail = end;  // before the whitespace that precedes </state>
      while (tail > e + 1 && is_space(text[tail - 1])) --tail;
      out += text.substr(q, e + 1 - q) + fr + text.substr(e + 1, tail - (e + 1)) + bk + text.substr(tail, end + 8 - tail);
      q = end + 8;
    }
    ++k;
  }
  if (k < front.size() || k < back.size()) throw Error(CG_ERR_INTERNAL, "xml: fewer <state> children than records");
  return out + text.substr(q);
}

std::string xml_append_attrs(const std::string& text, const std::string& tag, int index,
                             const std::vector<std::pair<std::string, std::string>>& attrs) {
  size_t p = 0;
  for (int i = 0;; ++i) {
    p = find_tag(text, tag, p, text.size());
    if (p == std::string::npos) throw Error(CG_ERR_PARSE, "xml: no <" + tag + "> number " + std::to_string(index));
    if (i == index) break;
    p = tag_end(text, p);
  }
  size_t e = tag_end(text, p);
  if (text[e - 1] == '/') --e;
  std::string add;
  for (auto& kv : attrs) add += " " + kv.first + "=\"" + kv.second + "\"";
  return text.substr(0, e) + add + text.substr(e);
}

std::string xlevels(const std::vector<std::string>& files, const std::string& out_xml) {
  // every state of every <nucleus> (else <system>) element of the files that
  // holds states (Xlevels includes each such space)
  std::vector<StateNode> all;
  for (const std::string& f : files) {
    std::ifstream in(f, std::ios::binary);
    if (!in) throw Error(CG_ERR_IO, "cannot open " + f);
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    std::string tag = find_tag(text, "nucleus", 0, text.size()) != std::string::npos ? "nucleus" : "system";
    size_t p = 0;
    while ((p = find_tag(text, tag, p, text.size())) != std::string::npos) {
      const size_t e = tag_end(text, p);
      if (text[e - 1] == '/') { p = e; continue; }
      const size_t close = text.find("</" + tag + ">", e);
      if (close == std::string::npos) throw Error(CG_ERR_PARSE, "xml: </" + tag + "> missing in " + f);
      std::string body = text.substr(e + 1, close - e - 1);
      std::vector<StateNode> st = take_states(body);
      for (auto& x : st) all.push_back(std::move(x));
      p = close;
    }
  }
  // OrganizeStates (include/xsm/xState.cxx:197-247): energy order, names
  // J P (k) per (J, P), Ex from the lowest
  std::vector<std::pair<double, size_t>> order;
  for (size_t i = 0; i < all.size(); ++i) {
    const std::string* E = get(all[i].attrs, "E");
    order.emplace_back(E ? std::atof(E->c_str()) : 0.0, i);
  }
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) { return a < b; });
  std::map<std::pair<std::string, std::string>, int> count;
  std::string listing, xml;
  std::vector<double> diff;
  for (auto& o : order) {
    StateNode& sn = all[o.second];
    const std::string* J = get(sn.attrs, "J");
    const std::string* P = get(sn.attrs, "P");
    std::string j = J ? *J : "??", pp = P ? *P : "?";
    const int k = ++count[{j, pp}];
    update(sn.attrs, "name", j + pp.substr(0, 1) + "(" + std::to_string(k) + ")");
    const double ex = o.first - order.front().first;
    update(sn.attrs, "Ex", num_str(ex));
    // ListStates (xmlshell/Xlevels.cpp:22-58): name T=.. Ex E [experimental Ex]
    const std::string* T = get(sn.attrs, "T");
    listing += *get(sn.attrs, "name") + " T=" + (T ? *T : std::string("???")) + " " + *get(sn.attrs, "Ex") + " " +
               num_str(o.first);
    bool data = false;
    for (const std::string& kid : sn.kids) {
      if (kid.compare(0, 5, "<data") || (kid.size() > 5 && !is_space(kid[5]) && kid[5] != '>' && kid[5] != '/'))
        continue;
      const Attrs da = parse_attrs(kid, 1, tag_end(kid, 0));
      if (const std::string* dx = get(da, "Ex")) {
        const double exd = std::atof(dx->c_str());
        listing += " " + num_str(exd);
        diff.push_back(std::atof(get(sn.attrs, "Ex")->c_str()) - exd);
        data = true;
      }
      break;
    }
    (void)data;
    listing += "\n";
    xml += "\n\t\t<state" + attrs_text(sn.attrs);
    if (sn.kids.empty()) {
      xml += "/>";
    } else {
      xml += ">";
      size_t wi = 0;
      for (const std::string& kid : sn.kids)
        xml += "\n\t\t\t" + (kid.empty() ? "<wavefunction" + attrs_text(sn.wfs[wi++]) + "/>" : kid);
      xml += "\n\t\t</state>";
    }
  }
  if (!diff.empty()) {
    double mean = 0.0, sig = 0.0;
    for (double d : diff) {
      mean += d;
      sig += d * d;
    }
    mean /= double(diff.size());
    listing += "Experimental data comparison\nMean (average shift) " + num_str(mean) + "\nRMS " +
               num_str(std::sqrt(sig / double(diff.size()) - mean * mean)) + "\n";
  }
  if (!out_xml.empty()) {
    std::ofstream of(out_xml, std::ios::binary);
    if (!of) throw Error(CG_ERR_IO, "cannot write " + out_xml);
    of << "<?xml version=\"1.0\"?>\n<cosmo>\n\t<nucleus>" << xml << "\n\t</nucleus>\n</cosmo>\n";
  }
  return listing;
}

std::string xml_add_states(const std::string& text, const std::string& system_name,
                           const std::vector<NewState>& add) {
  // the system element
  size_t sys = std::string::npos, p = 0;
  while ((p = find_tag(text, "system", p, text.size())) != std::string::npos) {
    const size_t e = tag_end(text, p);
    Attrs a = parse_attrs(text, p + 1, e);
    const std::string* nm = get(a, "name");
    if (system_name.empty() || (nm && *nm == system_name)) {
      sys = p;
      break;
    }
    p = e;
  }
  if (sys == std::string::npos) throw Error(CG_ERR_PARSE, "xml: system " + system_name + " not found");
  const size_t stag_end = tag_end(text, sys);
  std::string out;
  size_t body0, body1, after;
  std::string indent = "\t";
  {
    size_t ls = text.rfind('\n', sys);
    indent = text.substr(ls == std::string::npos ? 0 : ls + 1, sys - (ls == std::string::npos ? 0 : ls + 1));
    for (char& c : indent)
      if (!is_space(c)) c = ' ';
  }
  std::string head, body, tail;
  if (text[stag_end - 1] == '/') {  // <system .../> becomes <system ...> ... </system>
    head = text.substr(0, stag_end - 1) + ">";
    body = "";
    tail = "\n" + indent + "</system>" + text.substr(stag_end + 1);
  } else {
    body0 = stag_end + 1;
    body1 = text.find("</system>", body0);
    if (body1 == std::string::npos) throw Error(CG_ERR_PARSE, "xml: </system> missing");
    after = body1;
    head = text.substr(0, body0);
    body = text.substr(body0, body1 - body0);
    tail = text.substr(after);
  }
  // existing states, removed from the body
  std::vector<StateNode> states = take_states(body);
  // AddState: merge into a state with the same J, T and |dE| <= 0.001, else a new node
  for (const NewState& ns : add) {
    StateNode* hit = nullptr;
    for (auto& sn : states) {
      const std::string *J = get(sn.attrs, "J"), *T = get(sn.attrs, "T"), *E = get(sn.attrs, "E");
      if (!J || !T || !E) continue;
      if (parse_spin2(*J) != ns.twoJ || parse_spin2(*T) != ns.twoT) continue;
      if (std::fabs(std::atof(E->c_str()) - ns.E) > 0.001) continue;
      hit = &sn;
      break;
    }
    if (!hit) {
      states.emplace_back();
      hit = &states.back();
      update(hit->attrs, "name", spin_text(ns.twoJ));
      update(hit->attrs, "J", spin_text(ns.twoJ));
      update(hit->attrs, "P", ns.parity ? "-" : "+");
      update(hit->attrs, "T", spin_text(ns.twoT));
      hit->attrs.emplace_back("E", num_str(ns.E));
    }
    bool present = false;
    for (auto& wf : hit->wfs) {
      const std::string *f = get(wf, "file"), *id = get(wf, "id");
      if (f && *f == ns.file && id && std::atoi(id->c_str()) == ns.id) present = true;
    }
    if (!present) {
      Attrs wf;
      update(wf, "Jz", spin_text(ns.twoJz));
      update(wf, "Tz", spin_text(ns.twoTz));
      update(wf, "file", ns.file);
      update(wf, "id", std::to_string(ns.id));
      hit->wfs.push_back(wf);
      hit->kids.emplace_back();
    }
    update(hit->attrs, "dE", num_str(ns.dE));
  }
  // OrganizeStates: energy order, names J P (k) per (J, P), Ex from the lowest
  std::vector<std::pair<double, size_t>> order;
  for (size_t i = 0; i < states.size(); ++i) {
    const std::string* E = get(states[i].attrs, "E");
    order.emplace_back(E ? std::atof(E->c_str()) : 0.0, i);
  }
  std::stable_sort(order.begin(), order.end(),
                   [](const std::pair<double, size_t>& a, const std::pair<double, size_t>& b) { return a < b; });
  std::map<std::pair<std::string, std::string>, int> count;
  std::string emitted;
  const std::string in1 = indent + "\t", in2 = indent + "\t\t";
  for (auto& o : order) {
    StateNode& sn = states[o.second];
    const std::string* J = get(sn.attrs, "J");
    const std::string* P = get(sn.attrs, "P");
    std::string j = J ? *J : "??", pp = P ? *P : "?";
    int k = ++count[{j, pp}];
    update(sn.attrs, "name", j + pp.substr(0, 1) + "(" + std::to_string(k) + ")");
    update(sn.attrs, "Ex", num_str(o.first - order.front().first));
    emitted += "\n" + in1 + "<state" + attrs_text(sn.attrs);
    if (sn.kids.empty()) {
      emitted += "/>";
    } else {
      emitted += ">";
      size_t wi = 0;
      for (const std::string& kid : sn.kids)
        emitted += "\n" + in2 + (kid.empty() ? "<wavefunction" + attrs_text(sn.wfs[wi++]) + "/>" : kid);
      emitted += "\n" + in1 + "</state>";
    }
  }
  // keep the body's trailing whitespace before </system>
  size_t bt = body.size();
  while (bt > 0 && is_space(body[bt - 1])) --bt;
  std::string trail = body.substr(bt);
  if (trail.find('\n') == std::string::npos) trail = "\n" + indent;
  return head + body.substr(0, bt) + emitted + trail + tail;
}

std::vector<NewState> xshljt_states(const System& sys, const Basis& b, const std::string& ee_path, int nstates,
                                    const std::string& file_attr, std::vector<double>* jj_out,
                                    std::vector<double>* tt_out) {
  std::ifstream f(ee_path, std::ios::binary);
  if (!f) throw Error(CG_ERR_IO, "cannot open " + ee_path);
  uint32_t count = 0;
  f.read(reinterpret_cast<char*>(&count), 4);
  if (!f) throw Error(CG_ERR_IO, "short .EE file");
  uint32_t use = count;
  if (nstates > 0 && uint32_t(nstates) < count) use = uint32_t(nstates);
  std::vector<double> E(use), dE(use), vecs;
  vecs.resize(size_t(use) * b.n);
  for (uint32_t k = 0; k < use; ++k) {
    double dV;
    uint64_t n;
    f.read(reinterpret_cast<char*>(&E[k]), 8);
    f.read(reinterpret_cast<char*>(&dE[k]), 8);
    f.read(reinterpret_cast<char*>(&dV), 8);
    f.read(reinterpret_cast<char*>(&n), 8);
    if (!f || n != b.n) throw Error(CG_ERR_IO, ".EE vector dimension does not match the basis");
    f.read(reinterpret_cast<char*>(vecs.data() + size_t(k) * b.n), std::streamsize(n * 8));
    if (!f) throw Error(CG_ERR_IO, "short .EE file");
  }
  std::vector<double> jj(use), tt(use);
  for (uint32_t k0 = 0; k0 < use; k0 += 16) {
    const int m = int(std::min<uint32_t>(16, use - k0));
    jt_expectations(sys, b, vecs.data() + size_t(k0) * b.n, m, jj.data() + k0, tt.data() + k0);
  }
  const int two_tz = sys.nv - sys.zv;
  std::vector<NewState> out;
  for (uint32_t k = 0; k < use; ++k) {
    NewState s;
    s.twoJ = jj_spin(jj[k], sys.twom);
    if (sys.filter_twoJ >= 0 && s.twoJ != sys.filter_twoJ) continue;
    s.E = E[k];
    if (std::fabs(sys.jj) > 1e-8) s.E -= sys.jj * (double(s.twoJ - sys.twom) * double(s.twoJ + sys.twom + 2) / 4.0);
    s.twoT = jj_spin(tt[k], two_tz);
    if (sys.filter_twoT >= 0 && s.twoT != sys.filter_twoT) continue;
    s.dE = dE[k];
    s.parity = sys.parity;
    s.twoJz = sys.twom;
    s.twoTz = two_tz;
    s.file = file_attr;
    s.id = int(k);
    out.push_back(s);
  }
  if (jj_out) *jj_out = jj;
  if (tt_out) *tt_out = tt;
  return out;
}

}  // namespace cg
