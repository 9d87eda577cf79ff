// Shared helpers of the command-line drop-ins (argument parsing in the style of
// the reference's av::argparser: one positional file, single-letter flags with a
// value, and a few long options; status checking of C-ABI calls).
#pragma once
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "cosmo_gb300.h"

namespace cli {

struct Args {
  std::vector<std::string> pos;
  std::map<std::string, std::string> opt;  // "-n" -> "10", "--virtual" -> ""
  bool has(const std::string& k) const { return opt.count(k) != 0; }
  int geti(const std::string& k, int d) const { return has(k) ? std::atoi(opt.at(k).c_str()) : d; }
  double getd(const std::string& k, double d) const { return has(k) ? std::atof(opt.at(k).c_str()) : d; }
  std::string gets(const std::string& k, const std::string& d) const { return has(k) ? opt.at(k) : d; }
};

// flags listed in `with_value` take the next argument
inline Args parse(int argc, char** argv, const std::vector<std::string>& with_value) {
  Args a;
  for (int i = 1; i < argc; ++i) {
    std::string s = argv[i];
    if (s.size() > 1 && s[0] == '-') {
      bool v = false;
      for (auto& w : with_value) v = v || w == s;
      if (v) {
        if (i + 1 >= argc) {
          std::fprintf(stderr, "missing value for %s\n", s.c_str());
          std::exit(1);
        }
        a.opt[s] = argv[++i];
      } else {
        a.opt[s] = "";
      }
    } else {
      a.pos.push_back(s);
    }
  }
  return a;
}

inline void check(cg_status st, const char* what) {
  if (st != CG_OK) {
    std::fprintf(stderr, "%s failed (%d): %s\n", what, int(st), cg_last_error());
    std::exit(1);
  }
}

// the system name attribute of the selected (or only) <system> of an XML file
inline std::string system_name(const char* xml, const char* wanted) {
  if (wanted && *wanted) return wanted;
  FILE* f = std::fopen(xml, "rb");
  if (!f) return "system";
  std::string t;
  char buf[65536];
  size_t k;
  while ((k = std::fread(buf, 1, sizeof buf, f)) > 0) t.append(buf, k);
  std::fclose(f);
  size_t p = 0;
  while ((p = t.find("<system", p)) != std::string::npos) {
    char c = p + 7 < t.size() ? t[p + 7] : '>';
    if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '>') break;
    p += 7;
  }
  if (p == std::string::npos) return "system";
  size_t e = t.find('>', p);
  std::string tag = t.substr(p, e - p);
  size_t n = tag.find("name=");
  if (n == std::string::npos) return "system";
  char q = tag[n + 5];
  size_t v0 = n + 6, v1 = tag.find(q, v0);
  return tag.substr(v0, v1 - v0);
}

}  // namespace cli
