// Host-side problem setup: XML system subset, m-scheme s.p. table, Oxbash
// interaction reader and conversion to forward-ordered m-scheme operator
// terms (one-body ESP, two-body VSPX) including the lambda * J-J+ penalty.
//
// The conversion restates the reference's published formulas; each step cites
// the reference function it follows.  Values are FP64; TBMEs and s.p. energies
// are parsed as single precision exactly like the reference (std::stof).
#include "model.h"

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>

#include "cosmo_gb300.h"

namespace cg {

// ------------------------------------------------------------------ XML
const std::string* XmlNode::attr(const std::string& k) const {
  for (auto& a : attrs)
    if (a.first == k) return &a.second;
  return nullptr;
}
const XmlNode* XmlNode::child(const std::string& t, int index) const {
  int k = 0;
  for (auto& c : children)
    if (c.tag == t) {
      if (k == index) return &c;
      ++k;
    }
  return nullptr;
}
int XmlNode::count(const std::string& t) const {
  int k = 0;
  for (auto& c : children) k += (c.tag == t);
  return k;
}

namespace {
struct XmlReader {
  const std::string& s;
  size_t p = 0;
  explicit XmlReader(const std::string& str) : s(str) {}
  [[noreturn]] void fail(const std::string& m) {
    throw Error(CG_ERR_PARSE, "xml: " + m + " at offset " + std::to_string(p));
  }
  void ws() {
    while (p < s.size() && std::isspace((unsigned char)s[p])) ++p;
  }
  bool starts(const char* t) const { return s.compare(p, std::strlen(t), t) == 0; }
  void skip_misc() {
    for (;;) {
      ws();
      if (starts("<?")) {
        size_t e = s.find("?>", p);
        if (e == std::string::npos) fail("unterminated <?");
        p = e + 2;
      } else if (starts("<!--")) {
        size_t e = s.find("-->", p);
        if (e == std::string::npos) fail("unterminated comment");
        p = e + 3;
      } else if (starts("<!")) {
        size_t e = s.find('>', p);
        if (e == std::string::npos) fail("unterminated <!");
        p = e + 1;
      } else {
        return;
      }
    }
  }
  static std::string unescape(const std::string& v) {
    std::string o;
    for (size_t i = 0; i < v.size(); ++i) {
      if (v[i] == '&') {
        size_t e = v.find(';', i);
        if (e != std::string::npos) {
          std::string ent = v.substr(i + 1, e - i - 1);
          const char* r = nullptr;
          if (ent == "amp") r = "&"; else if (ent == "lt") r = "<"; else if (ent == "gt") r = ">";
          else if (ent == "quot") r = "\""; else if (ent == "apos") r = "'";
          if (r) { o += r; i = e; continue; }
        }
      }
      o += v[i];
    }
    return o;
  }
  std::string name() {
    size_t b = p;
    while (p < s.size() && !std::isspace((unsigned char)s[p]) && s[p] != '>' && s[p] != '/' && s[p] != '=')
      ++p;
    if (p == b) fail("expected a name");
    return s.substr(b, p - b);
  }
  XmlNode element() {
    if (p >= s.size() || s[p] != '<') fail("expected '<'");
    ++p;
    XmlNode n;
    n.tag = name();
    for (;;) {
      ws();
      if (p >= s.size()) fail("unterminated tag");
      if (s[p] == '/') {
        if (p + 1 >= s.size() || s[p + 1] != '>') fail("bad '/'");
        p += 2;
        return n;
      }
      if (s[p] == '>') { ++p; break; }
      std::string k = name();
      ws();
      if (p >= s.size() || s[p] != '=') fail("expected '=' after attribute " + k);
      ++p;
      ws();
      char q = s[p];
      if (q != '"' && q != '\'') fail("expected quote");
      size_t e = s.find(q, p + 1);
      if (e == std::string::npos) fail("unterminated attribute");
      n.attrs.emplace_back(k, unescape(s.substr(p + 1, e - p - 1)));
      p = e + 1;
    }
    for (;;) {
      size_t b = p;
      while (p < s.size() && s[p] != '<') ++p;
      n.text += unescape(s.substr(b, p - b));
      if (p >= s.size()) fail("unterminated element " + n.tag);
      if (starts("</")) {
        p += 2;
        std::string t = name();
        if (t != n.tag) fail("mismatched </" + t + "> for <" + n.tag + ">");
        ws();
        if (p >= s.size() || s[p] != '>') fail("expected '>'");
        ++p;
        break;
      }
      if (starts("<?") || starts("<!")) {
        skip_misc();
        continue;
      }
      n.children.push_back(element());
    }
    // trim text
    size_t a = n.text.find_first_not_of(" \t\r\n");
    size_t z = n.text.find_last_not_of(" \t\r\n");
    n.text = (a == std::string::npos) ? std::string() : n.text.substr(a, z - a + 1);
    return n;
  }
};
}  // namespace

XmlNode parse_xml_file(const std::string& path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(CG_ERR_IO, "cannot open " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  std::string s = ss.str();
  if (s.size() >= 3 && (unsigned char)s[0] == 0xEF && (unsigned char)s[1] == 0xBB && (unsigned char)s[2] == 0xBF)
    s = s.substr(3);
  XmlReader r(s);
  r.skip_misc();
  return r.element();
}

// ------------------------------------------------------------ numbers
// Doubled spin from text: "5/2" -> 5, "3" -> 6, "1.5" -> 3, as the reference
// `spin(const char*)` constructor (include/sm/spinclass.cxx:57-79).
int parse_spin2(const std::string& t) {
  size_t sl = t.find('/');
  if (sl != std::string::npos) {
    if (t.substr(sl + 1) != "2") throw Error(CG_ERR_PARSE, "bad spin " + t);
    return std::atoi(t.substr(0, sl).c_str());
  }
  double x = std::atof(t.c_str());
  int r = x >= 0 ? int(2.0 * x + 0.5) : int(2.0 * x - 0.5);
  if (std::fabs(r - 2.0 * x) > 0.01) throw Error(CG_ERR_PARSE, "spin " + t + " is not (half-)integer");
  return r;
}
namespace {
int attr_int(const XmlNode& n, const char* k, int dflt, bool required = false) {
  const std::string* v = n.attr(k);
  if (!v) {
    if (required) throw Error(CG_ERR_PARSE, std::string("missing attribute ") + k + " on <" + n.tag + ">");
    return dflt;
  }
  return std::atoi(v->c_str());
}
std::string dirname_of(const std::string& p) {
  size_t s = p.find_last_of('/');
  return s == std::string::npos ? std::string(".") : p.substr(0, s);
}
bool file_exists(const std::string& p) {
  std::ifstream f(p);
  return bool(f);
}
}  // namespace

// --------------------------------------------------------- system + sps
// Follows SM::Make(sps, XMLNode) (include/xsm/xSingleParticleStates.cxx:26-104):
// orbitals sorted by their `index`, m = -j..j, neutron copies first, then
// proton copies (lines 100-101).  The system attributes follow
// SM::MakeMBS2(XMLNode, sps) (include/xsm/xManyBodyStates.cxx:22-91).
System load_system(const std::string& xml_path, const std::string& system_name) {
  XmlNode root = parse_xml_file(xml_path);
  if (root.tag != "cosmo") throw Error(CG_ERR_PARSE, "root element is <" + root.tag + ">, expected <cosmo>");
  System sys;
  sys.xml_dir = dirname_of(xml_path);
  const XmlNode* vs = root.child("valencespace");
  if (!vs) throw Error(CG_ERR_PARSE, "no <valencespace>");
  std::map<int, const XmlNode*> by_index;
  for (auto& c : vs->children)
    if (c.tag == "orbital") by_index[attr_int(c, "index", 0, true)] = &c;
  if (by_index.empty()) throw Error(CG_ERR_PARSE, "no orbitals defined");
  std::vector<SPState> neutrons, protons;
  for (auto& kv : by_index) {
    const XmlNode& o = *kv.second;
    Orbit ob;
    ob.index = kv.first;
    ob.name = o.attr("name") ? *o.attr("name") : std::string();
    if (!o.attr("j")) throw Error(CG_ERR_PARSE, "orbital without j");
    ob.j2 = parse_spin2(*o.attr("j"));
    ob.n = attr_int(o, "n", 0);
    ob.l = attr_int(o, "l", 0);
    ob.parity = ob.l & 1;
    if (const std::string* pp = o.attr("P")) ob.parity = (*pp == "-" || *pp == "1") ? 1 : 0;
    ob.t2 = 1;
    if (const std::string* tt = o.attr("T")) ob.t2 = parse_spin2(*tt);
    if (ob.t2 != 1) throw Error(CG_ERR_UNSUPPORTED, "only isospin-1/2 orbitals are supported");
    ob.type = o.attr("type") ? *o.attr("type") : std::string("pn");
    if (ob.type != "pn" && ob.type != "p" && ob.type != "n")
      throw Error(CG_ERR_PARSE, "orbital type must be pn, p or n");
    sys.orbits.push_back(ob);
    for (int m = -ob.j2; m <= ob.j2; m += 2) {
      SPState x{ob.index - 1, ob.n, ob.l, ob.j2, m, ob.t2, 0, ob.parity};
      if (ob.type == "pn" || ob.type == "n") { x.tz2 = 1; neutrons.push_back(x); }
      if (ob.type == "pn" || ob.type == "p") { x.tz2 = -1; protons.push_back(x); }
    }
  }
  sys.sps = neutrons;
  sys.sps.insert(sys.sps.end(), protons.begin(), protons.end());
  sys.n_neutron_states = int(neutrons.size());
  // up to 64 m-states per species (masks of one 64-bit word per species)
  if (sys.n_neutron_states > 64 || int(sys.sps.size()) - sys.n_neutron_states > 64)
    throw Error(CG_ERR_UNSUPPORTED, "more than 64 m-scheme s.p. states per species");

  // system node
  const XmlNode* sn = nullptr;
  int nsys = root.count("system");
  if (nsys == 0) throw Error(CG_ERR_PARSE, "no <system>");
  if (!system_name.empty()) {
    for (int i = 0; i < nsys; ++i) {
      const XmlNode* c = root.child("system", i);
      if (c->attr("name") && *c->attr("name") == system_name) sn = c;
    }
    if (!sn) throw Error(CG_ERR_ARG, "no <system name=\"" + system_name + "\">");
  } else {
    if (nsys > 1) throw Error(CG_ERR_ARG, "several <system> nodes: give a system name");
    sn = root.child("system");
  }
  sys.name = sn->attr("name") ? *sn->attr("name") : std::string("system");
  int A = attr_int(*sn, "Av", 0, true);
  if (sn->attr("Nv") && sn->attr("Zv")) {
    sys.nv = attr_int(*sn, "Nv", 0);
    sys.zv = attr_int(*sn, "Zv", 0);
  } else if (sn->attr("Tz")) {
    int tz2 = parse_spin2(*sn->attr("Tz"));
    sys.zv = (A - tz2) / 2;
    sys.nv = (A + tz2) / 2;
  } else {
    throw Error(CG_ERR_PARSE, "system needs Nv/Zv or Tz");
  }
  if (sys.nv + sys.zv != A) throw Error(CG_ERR_PARSE, "Nv + Zv != Av");
  sys.twom = sn->attr("Jz") ? parse_spin2(*sn->attr("Jz")) : (A % 2);
  if (const std::string* fj = sn->attr("J")) sys.filter_twoJ = parse_spin2(*fj);
  if (const std::string* ft = sn->attr("T")) sys.filter_twoT = parse_spin2(*ft);
  if (!sn->attr("P")) throw Error(CG_ERR_PARSE, "system needs P");
  sys.parity = ((*sn->attr("P"))[0] == '-') ? 1 : 0;
  // basis truncation (XsysmbsOMP, xmlshell/xmbs/XsysmbsOMP.cpp:214-300); the
  // reference's getXMLData (include/xmlParser.cxx:129) reads a value from an
  // attribute or from the text of a child element
  auto xml_value = [](const XmlNode& nd, const char* k) -> const std::string* {
    if (const std::string* a = nd.attr(k)) return a;
    if (const XmlNode* c = nd.child(k)) return &c->text;
    return nullptr;
  };
  auto xml_int = [&](const XmlNode& nd, const char* k) {
    const std::string* v = xml_value(nd, k);
    if (!v) throw Error(CG_ERR_PARSE, std::string("missing ") + k + " on <" + nd.tag + ">");
    return std::atoi(v->c_str());
  };
  if (const std::string* hm = xml_value(*sn, "hwmax")) {
    sys.trunc.hw = true;
    sys.trunc.hwmax = std::atoi(hm->c_str());
    sys.trunc.hwmin = 0;
    sys.truncation += "hwmax ";
  }
  if (const XmlNode* hr = sn->child("hwrejection")) {  // only the first one counts, as in the reference
    sys.trunc.hw = true;
    sys.trunc.hwmax = xml_int(*hr, "HWMAX");
    sys.trunc.hwmin = xml_int(*hr, "HWMIN");
    sys.truncation += "<hwrejection> ";
  }
  for (int r = 0; r < sn->count("rejection"); ++r) {
    const XmlNode* rj = sn->child("rejection", r);
    Truncation::Rejection rej;
    rej.nmin = xml_int(*rj, "NMIN");
    rej.nmax = xml_int(*rj, "NMAX");
    for (int o = 0; o < rj->count("orbital"); ++o) {
      const XmlNode* ob = rj->child("orbital", o);
      const int level = xml_int(*ob, "index") - 1;
      const std::string type = ob->attr("type") ? *ob->attr("type") : std::string("n");
      for (size_t i = 0; i < sys.sps.size(); ++i) {
        const bool neut = sys.sps[i].tz2 > 0;
        if (sys.sps[i].level == level && ((neut && (type == "pn" || type == "n")) || (!neut && (type == "pn" || type == "p")))) {
          if (i < 64) rej.mask |= 1ull << i;
          if (int(i) < sys.n_neutron_states) rej.nmask |= 1ull << i;
          else rej.pmask |= 1ull << (i - sys.n_neutron_states);
        }
      }
    }
    sys.trunc.rejections.push_back(rej);
    if (r == 0) sys.truncation += "<rejection> ";
  }
  if (const XmlNode* mb = sn->child("ManyBodyStates"))
    if (mb->attr("name")) sys.mbs_name = *mb->attr("name");
  if (const XmlNode* mx = sn->child("matrix")) {
    if (mx->attr("JJ")) {
      sys.has_jj = true;
      sys.jj = std::atof(mx->attr("JJ")->c_str());
    }
    if (mx->attr("TT")) throw Error(CG_ERR_UNSUPPORTED, "matrix TT term is not supported");
  }
  // interaction files (ReadXMLINT, include/xsm/xsphericalint.cxx:16-49)
  const XmlNode* hn = root.child("hamiltonian");
  if (!hn) throw Error(CG_ERR_PARSE, "no <hamiltonian>");
  int nf = hn->count("file");
  if (nf == 0) throw Error(CG_ERR_UNSUPPORTED, "only Oxbash <file> interactions are supported");
  for (int i = 0; i < nf; ++i) {
    const XmlNode* fn = hn->child("file", i);
    const XmlNode* nm = fn->child("name");
    if (!nm) throw Error(CG_ERR_PARSE, "<file> without <name>");
    std::array<double, 10> sc;
    sc.fill(1.0);
    for (int s = 0; s < fn->count("scale"); ++s) {
      const XmlNode* sx = fn->child("scale", s);
      int rank = attr_int(*sx, "rank", 0, true);
      if (rank < 0 || rank > 9) throw Error(CG_ERR_PARSE, "bad scale rank");
      sc[rank] *= std::atof(sx->text.c_str());
    }
    sys.int_files.push_back(nm->text);
    sys.int_scale.push_back(sc);
  }
  return sys;
}

// ----------------------------------------------------- Oxbash reader
namespace {
std::string resolve_int(const System& sys, const std::string& name) {
  std::vector<std::string> cands;
  const char* env = std::getenv("SMINTPATH");
  auto add = [&](const std::string& base) {
    cands.push_back(base);
    cands.push_back(base + ".int");
  };
  add(name);
  if (!name.empty() && name[0] != '/') {
    add(sys.xml_dir + "/" + name);
    if (env) {
      std::string paths = env;
      size_t b = 0;
      while (b <= paths.size()) {
        size_t e = paths.find_first_of(":;", b);
        if (e == std::string::npos) e = paths.size();
        if (e > b) add(paths.substr(b, e - b) + "/" + name);
        b = e + 1;
      }
    }
  }
  for (auto& c : cands)
    if (file_exists(c)) return c;
  throw Error(CG_ERR_IO, "interaction file not found: " + name);
}

bool comment_line(const std::string& l) {
  // av::CommentString (include/av/TextAnalysis.cxx:31-39): leading '#', '!', '%' or '/'
  size_t p = l.find_first_not_of(' ');
  if (p == std::string::npos) return false;
  return std::strchr("#!%/", l[p]) != nullptr && l[p] != '\0';
}

std::vector<std::string> split_tokens(const std::string& l) {
  std::vector<std::string> t;
  std::string cur;
  for (char c : l) {
    if (std::isspace((unsigned char)c) || c == ',') {
      if (!cur.empty()) t.push_back(cur), cur.clear();
    } else {
      cur += c;
    }
  }
  if (!cur.empty()) t.push_back(cur);
  return t;
}

// CheckSphericalINT (include/sm/sphericalint.cxx:43-84): a later line that
// repeats an earlier one (same sorted pairs, possibly bra <-> ket swapped, same
// J and T) is zeroed.
void zero_repeated(std::map<std::array<int, 6>, double>& t) {
  for (auto i1 = t.begin(); i1 != t.end(); ++i1) {
    int a[4];
    const auto& k1 = i1->first;
    if (k1[0] < k1[1]) { a[0] = k1[0]; a[1] = k1[1]; } else { a[1] = k1[0]; a[0] = k1[1]; }
    if (k1[2] < k1[3]) { a[2] = k1[2]; a[3] = k1[3]; } else { a[2] = k1[3]; a[3] = k1[2]; }
    auto i2 = i1;
    for (++i2; i2 != t.end(); ++i2) {
      const auto& k2 = i2->first;
      if (k1[4] != k2[4] || k1[5] != k2[5]) continue;
      int b[4];
      if (k2[0] < k2[1]) { b[0] = k2[0]; b[1] = k2[1]; } else { b[1] = k2[0]; b[0] = k2[1]; }
      if (k2[2] < k2[3]) { b[2] = k2[2]; b[3] = k2[3]; } else { b[2] = k2[3]; b[3] = k2[2]; }
      bool bad = (a[0] == b[0] && a[1] == b[1] && a[2] == b[2] && a[3] == b[3]) ||
                 (a[0] == b[2] && a[1] == b[3] && a[2] == b[0] && a[3] == b[1]);
      if (bad) i2->second = 0.0;
    }
  }
}
}  // namespace

// ReadOxbashINT (include/sm/sphericalint.cxx:145-246) for every <file>.
SphericalInt read_oxbash(const System& sys) {
  SphericalInt out;
  int A = sys.nv + sys.zv;
  for (size_t fi = 0; fi < sys.int_files.size(); ++fi) {
    std::string path = resolve_int(sys, sys.int_files[fi]);
    std::ifstream f(path);
    if (!f) throw Error(CG_ERR_IO, "cannot open " + path);
    double spescaling = sys.int_scale[fi][1], vscaling = sys.int_scale[fi][2];
    std::map<std::array<int, 6>, double> tmp;
    std::string line;
    int linecount = 0;
    while (std::getline(f, line)) {
      if (!line.empty() && line.back() == '\r') line.pop_back();
      if (line.empty()) continue;
      size_t p = line.find_first_not_of(" \t\n\v\f\r");
      line = (p == std::string::npos) ? std::string() : line.substr(p);
      if (comment_line(line)) continue;
      std::vector<std::string> tok = split_tokens(line);
      try {
        if (linecount == 0) {
          int intlines = std::stoi(tok.at(0));
          int words = int(tok.size()) - 1;
          if (intlines < 0) words -= 3;
          if (words < 0) throw Error(CG_ERR_PARSE, "bad first line in " + path);
          if (int(out.spe.size()) < words) out.spe.resize(words, 0.0);
          for (int i = 0; i < words; ++i) out.spe[i] += std::stof(tok[i + 1]) * spescaling;
          if (intlines < 0) {
            double acore = std::stof(tok.at(words + 1));
            double ascale = std::stof(tok.at(words + 2));
            double spow = std::stof(tok.at(words + 3));
            if (A >= 0) vscaling *= std::pow(ascale / (A + acore), spow);
          }
        } else {
          if (tok.size() < 7) { ++linecount; continue; }
          std::array<int, 6> ijk;
          ijk[2] = std::stoi(tok[0]) - 1;
          ijk[3] = std::stoi(tok[1]) - 1;
          ijk[0] = std::stoi(tok[2]) - 1;
          ijk[1] = std::stoi(tok[3]) - 1;
          ijk[4] = std::stoi(tok[4]);
          ijk[5] = std::stoi(tok[5]);
          tmp[ijk] += vscaling * double(std::stof(tok[6]));
        }
      } catch (const Error&) {
        throw;
      } catch (const std::exception&) {
        throw Error(CG_ERR_PARSE, "cannot parse line in " + path + ": " + line);
      }
      ++linecount;
    }
    zero_repeated(tmp);
    for (auto& kv : tmp) {
      if (kv.first[5] < 0) throw Error(CG_ERR_UNSUPPORTED, "Tz-resolved interactions are not supported");
      out.tbme[kv.first] += kv.second;
    }
  }
  return out;
}

// ------------------------------------------------------ Clebsch-Gordan
// Racah's closed formula, doubled arguments.
namespace {
long double fact(int n) {
  static long double tab[64];
  static bool init = false;
  if (!init) {
    tab[0] = 1.0L;
    for (int i = 1; i < 64; ++i) tab[i] = tab[i - 1] * i;
    init = true;
  }
  return tab[n];
}
}  // namespace

double clebsch_gordan(int j1, int m1, int j2, int m2, int j3, int m3) {
  if (m1 + m2 != m3) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  if (((j1 + m1) & 1) || ((j2 + m2) & 1) || ((j3 + m3) & 1)) return 0.0;
  if (j3 > j1 + j2 || j3 < std::abs(j1 - j2) || ((j1 + j2 + j3) & 1)) return 0.0;
  int a = (j1 + j2 - j3) / 2, b = (j1 - j2 + j3) / 2, c = (-j1 + j2 + j3) / 2, d = (j1 + j2 + j3) / 2 + 1;
  long double delta = fact(a) * fact(b) * fact(c) / fact(d);
  long double pre = std::sqrt((long double)(j3 + 1) * delta * fact((j1 + m1) / 2) * fact((j1 - m1) / 2) *
                              fact((j2 + m2) / 2) * fact((j2 - m2) / 2) * fact((j3 + m3) / 2) *
                              fact((j3 - m3) / 2));
  long double sum = 0.0L;
  for (int k = 0; k <= d; ++k) {
    int e1 = (j1 + j2 - j3) / 2 - k, e2 = (j1 - m1) / 2 - k, e3 = (j2 + m2) / 2 - k;
    int e4 = (j3 - j2 + m1) / 2 + k, e5 = (j3 - j1 - m2) / 2 + k;
    if (e1 < 0 || e2 < 0 || e3 < 0 || e4 < 0 || e5 < 0) continue;
    long double term = 1.0L / (fact(k) * fact(e1) * fact(e2) * fact(e3) * fact(e4) * fact(e5));
    sum += (k & 1) ? -term : term;
  }
  return double(pre * sum);
}

// -------------------------------------------------- m-scheme operator
namespace {
// AddPPVsp, 4-argument form (include/sm/AddPPVsp.cxx:32-147): every m-state
// combination of the four orbits, Clebsch-Gordan weights in J and T,
// 1/sqrt((1+d_ab)(1+d_cd)), sqrt(2) for pn pairs of separately indexed orbits,
// fermion sign on pair reordering, forward pair order, /2 for a line whose bra
// and ket orbit pairs coincide and x2 on the m-pair diagonal.
// Clebsch-Gordan coefficients <j1 m1 j2 m2 | J m1+m2> of two s.p. states
// (odd doubled j1, j2 <= jmax) and of their isospins (t = 1/2), tabulated once
// per operator build from clebsch_gordan itself (same values, looked up
// instead of recomputed for every m-state combination of every TBME line).
struct CGTable {
  int jmax = 0, nj = 0, nm = 0;
  std::vector<double> tab;  // [j1][m1][j2][m2][J]
  double tz[2][2][2];       // [tz1 > 0][tz2 > 0][T]
  explicit CGTable(int jmax_) : jmax(jmax_ | 1), nj((jmax_ + 2) / 2), nm(jmax_ + 2) {
    const int nJ = nm;
    tab.assign(size_t(nj) * nm * nj * nm * nJ, 0.0);
    for (int a = 0; a < nj; ++a)
      for (int b = 0; b < nj; ++b) {
        const int j1 = 2 * a + 1, j2 = 2 * b + 1;
        for (int m1 = -j1; m1 <= j1; m1 += 2)
          for (int m2 = -j2; m2 <= j2; m2 += 2)
            for (int J = std::abs(j1 - j2); J <= j1 + j2 && J / 2 < nJ; J += 2)
              tab[idx(j1, m1, j2, m2, J)] = clebsch_gordan(j1, m1, j2, m2, J, m1 + m2);
      }
    for (int p = 0; p < 2; ++p)
      for (int q = 0; q < 2; ++q)
        for (int T = 0; T < 2; ++T) tz[p][q][T] = clebsch_gordan(1, p ? 1 : -1, 1, q ? 1 : -1, 2 * T, (p ? 1 : -1) + (q ? 1 : -1));
  }
  size_t idx(int j1, int m1, int j2, int m2, int J) const {
    return (((size_t(j1 / 2) * nm + (m1 + jmax) / 2) * nj + j2 / 2) * nm + (m2 + jmax) / 2) * nm + J / 2;
  }
  double j(int j1, int m1, int j2, int m2, int J) const {
    if ((j1 & 1) == 0 || (j2 & 1) == 0 || (J & 1) || J / 2 >= nm || j1 > jmax || j2 > jmax)
      return clebsch_gordan(j1, m1, j2, m2, J, m1 + m2);
    return tab[idx(j1, m1, j2, m2, J)];
  }
  double t(int tz1, int tz2, int T) const {
    if (T < 0 || T > 1) return clebsch_gordan(1, tz1, 1, tz2, 2 * T, tz1 + tz2);
    return tz[tz1 > 0][tz2 > 0][T];
  }
};

// s.p. indices of each orbit level (ascending; both species), and the index
// of (level, tz, m) for the direct lookup of the fourth state of a TBME term
struct SPIndex {
  int jmax = 1;
  std::vector<std::vector<int>> by_level;
  std::vector<int> at;  // [level][tz > 0][(m + jmax) / 2] -> index or -1
  explicit SPIndex(const std::vector<SPState>& sps) {
    int nl = 0;
    for (const auto& sp : sps) {
      nl = std::max(nl, sp.level + 1);
      jmax = std::max(jmax, sp.j2);
    }
    by_level.assign(nl, {});
    at.assign(size_t(nl) * 2 * (jmax + 1), -1);
    for (int i = 0; i < int(sps.size()); ++i) {
      by_level[sps[i].level].push_back(i);
      at[slot(sps[i].level, sps[i].tz2, sps[i].m2)] = i;
    }
  }
  size_t slot(int level, int tz2, int m2) const {
    return (size_t(level) * 2 + (tz2 > 0)) * (jmax + 1) + (m2 + jmax) / 2;
  }
  int find(int level, int tz2, int m2) const {
    if (level < 0 || level >= int(by_level.size()) || m2 < -jmax || m2 > jmax || (tz2 != 1 && tz2 != -1)) return -1;
    return at[slot(level, tz2, m2)];
  }
};

// AddPPVsp, 4-argument form (include/sm/AddPPVsp.cxx:32-147): every m-state
// combination of the four orbits, Clebsch-Gordan weights in J and T,
// 1/sqrt((1+d_ab)(1+d_cd)), sqrt(2) for pn pairs of separately indexed orbits,
// fermion sign on pair reordering, forward pair order, /2 for a line whose bra
// and ket orbit pairs coincide and x2 on the m-pair diagonal.  The states are
// visited in ascending index order as in the reference (a0, a1, a2; the fourth
// is fixed by m and tz conservation), so every key accumulates its terms in
// the reference's order.
void add_pp_vsp(std::map<Key4, double>& vsp, const std::vector<SPState>& sps, const CGTable& cgt,
                const SPIndex& spi, const std::array<int, 6>& ijk, double V) {
  const int nl = int(spi.by_level.size());
  for (int q = 0; q < 4; ++q)
    if (ijk[q] < 0 || ijk[q] >= nl || spi.by_level[ijk[q]].empty()) return;
  const int l2 = sps[spi.by_level[ijk[1]][0]].j2, l3 = 2 * ijk[4];
  for (int a0 : spi.by_level[ijk[0]]) {
    const int l1 = sps[a0].j2, m1 = sps[a0].m2;
    for (int a1 : spi.by_level[ijk[1]]) {
      if ((sps[a0].j2 & 1) && a1 == a0) continue;
      const int m2 = sps[a1].m2;
      const double cg_ab = cgt.j(l1, m1, l2, m2, l3);
      for (int a2 : spi.by_level[ijk[2]]) {
        const int a3 = spi.find(ijk[3], sps[a0].tz2 + sps[a1].tz2 - sps[a2].tz2,
                                sps[a0].m2 + sps[a1].m2 - sps[a2].m2);
        if (a3 < 0) continue;
        if ((sps[a2].j2 & 1) && a2 == a3) continue;
        double h = cg_ab;
        h *= cgt.j(sps[a2].j2, sps[a2].m2, sps[a3].j2, sps[a3].m2, l3);
        if (sps[a0].t2 == 1 && sps[a1].t2 == 1 && sps[a2].t2 == 1 && sps[a3].t2 == 1) {
          h *= cgt.t(sps[a0].tz2, sps[a1].tz2, ijk[5]);
          h *= cgt.t(sps[a2].tz2, sps[a3].tz2, ijk[5]);
        } else {
          h *= clebsch_gordan(sps[a0].t2, sps[a0].tz2, sps[a1].t2, sps[a1].tz2, 2 * ijk[5],
                              sps[a0].tz2 + sps[a1].tz2);
          h *= clebsch_gordan(sps[a2].t2, sps[a2].tz2, sps[a3].t2, sps[a3].tz2, 2 * ijk[5],
                              sps[a2].tz2 + sps[a3].tz2);
        }
        if (std::fabs(h) < 1e-9) continue;
        h = h * V / std::sqrt((double(ijk[0] == ijk[1]) + 1.) * (double(ijk[2] == ijk[3]) + 1.));
        auto pn_pair = [&](int x, int y) {
          return sps[x].n == sps[y].n && sps[x].j2 == sps[y].j2 && sps[x].tz2 == -sps[y].tz2 &&
                 sps[x].parity == sps[y].parity;
        };
        if (ijk[0] != ijk[1] && pn_pair(a0, a1)) h *= std::sqrt(2.);
        if (ijk[2] != ijk[3] && pn_pair(a2, a3)) h *= std::sqrt(2.);
        Key4 bk{a0, a1, a2, a3};
        bool phase = false;
        if (bk[0] > bk[1]) { std::swap(bk[0], bk[1]); phase ^= bool(sps[a0].j2 & 1); }
        if (bk[2] > bk[3]) { std::swap(bk[2], bk[3]); phase ^= bool(sps[a2].j2 & 1); }
        if (bk[2] < bk[0] || (bk[2] == bk[0] && bk[3] < bk[1])) { std::swap(bk[0], bk[2]); std::swap(bk[1], bk[3]); }
        if (ijk[0] == ijk[2] && ijk[1] == ijk[3]) h /= 2.0;
        if (bk[0] == bk[2] && bk[1] == bk[3]) h *= 2.0;
        vsp[bk] += phase ? -h : h;
      }
    }
  }
}

// SPJPlus (include/sm/spherical2sp.cxx:629-659): one-body J+ with
// q = sqrt((j-m)(j+m+1)) on (jm -> jm+1), keyed (annihilated, created).
std::map<Key2, double> j_plus(const std::vector<SPState>& sps) {
  std::map<Key2, double> jo;
  const int ns = int(sps.size());
  for (int p0 = 0; p0 < ns; ++p0)
    for (int p1 = p0 + 1; p1 < ns; ++p1) {
      const SPState &s0 = sps[p0], &s1 = sps[p1];
      if (s0.level != s1.level || s0.tz2 != s1.tz2) continue;
      if (s0.m2 + 2 == s1.m2)
        jo[{p0, p1}] = std::sqrt((s0.j2 - s0.m2) * (s0.j2 + s0.m2 + 2.)) / 2.0;
      else if (s0.m2 - 2 == s1.m2)
        jo[{p1, p0}] = std::sqrt((s1.j2 - s1.m2) * (s1.j2 + s1.m2 + 2.)) / 2.0;
    }
  return jo;
}

// SPSqrM (include/sm/cioperators.cxx:200-240) followed by
// StripHermitianOperator (:274-287): J-J+ as one-body (from the
// anticommutator) plus two-body terms, then only forward keys are kept.
void j_minus_j_plus(const std::map<Key2, double>& jo, std::map<Key2, double>& jsp,
                    std::map<Key4, double>& vsp) {
  for (auto& i : jo)
    for (auto& j : jo) {
      double h = i.second * j.second;
      if (std::fabs(h) < 1e-8) continue;
      if (j.first[1] == i.first[1]) jsp[{j.first[0], i.first[0]}] += h;
      Key4 aa{j.first[1], i.first[0], j.first[0], i.first[1]};
      if (aa[0] > aa[1]) { std::swap(aa[0], aa[1]); h = -h; }
      if (aa[2] > aa[3]) { std::swap(aa[2], aa[3]); h = -h; }
      vsp[aa] += h;
    }
  for (auto it = jsp.begin(); it != jsp.end();) {
    if (it->first[1] < it->first[0]) it = jsp.erase(it); else ++it;
  }
  for (auto it = vsp.begin(); it != vsp.end();) {
    const Key4& k = it->first;
    bool backward = (k[2] < k[0]) || (k[2] == k[0] && k[3] < k[1]);
    if (backward) it = vsp.erase(it); else ++it;
  }
}
}  // namespace

std::map<Key2, double> j_plus_terms(const std::vector<SPState>& sps) { return j_plus(sps); }

std::map<Key2, double> t_plus_terms(const System& sys) {
  std::map<Key2, double> to;
  const int nn = sys.n_neutron_states, ns = int(sys.sps.size());
  for (int y = 0; y < nn; ++y)
    for (int x = nn; x < ns; ++x) {
      const SPState &X = sys.sps[x], &Y = sys.sps[y];
      if (X.level == Y.level && X.m2 == Y.m2 && X.n == Y.n && X.l == Y.l && X.j2 == Y.j2 && X.parity == Y.parity &&
          X.t2 == Y.t2 && X.tz2 + 2 == Y.tz2)
        to[{x, y}] = std::sqrt(double(X.t2 - X.tz2) * double(X.t2 + X.tz2 + 2)) / 2.0;
    }
  return to;
}

Operator square_operator(const std::map<Key2, double>& raise) {
  Operator op;
  j_minus_j_plus(raise, op.one, op.two);
  return op;
}

// xReadSPInt, Oxbash branch + JJ branch (include/xsm/xReadSPInt.cxx:58-73,
// 273-287): ESP from the s.p. energies (MakeESPO, include/sm/MakeSPO.cxx:195),
// VSPX from every TBME line (PPInteraction2sp, include/sm/spherical2sp.cxx:790),
// then ESP += lambda*JSP and VSPX += lambda*SPJJ.
Operator build_operator(const System& sys) {
  SphericalInt si = read_oxbash(sys);
  Operator op;
  const int ns = int(sys.sps.size());
  for (int i = 0; i < ns; ++i) {
    int lv = sys.sps[i].level;
    if (lv >= int(si.spe.size())) throw Error(CG_ERR_PARSE, "interaction has fewer s.p. energies than orbits");
    op.one[{i, i}] += si.spe[lv];
  }
  int jmax = 1;
  for (const auto& sp : sys.sps) jmax = std::max(jmax, sp.j2);
  const CGTable cgt(jmax);
  const SPIndex spi(sys.sps);
  for (auto& kv : si.tbme) add_pp_vsp(op.two, sys.sps, cgt, spi, kv.first, kv.second);
  if (sys.has_jj) {
    std::map<Key2, double> jsp;
    std::map<Key4, double> vjj;
    j_minus_j_plus(j_plus(sys.sps), jsp, vjj);
    for (auto& kv : jsp) op.one[kv.first] += kv.second * sys.jj;
    for (auto& kv : vjj) op.two[kv.first] += kv.second * sys.jj;
  }
  return op;
}

}  // namespace cg
