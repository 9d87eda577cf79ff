// Drop-in for XSHLEMB (xmlshell/XSHLEMB.cpp:116-372): electric, magnetic,
// Gamow-Teller and Fermi transition rates between the <state>s of a parent
// system and those of a daughter system, for the <operator> node of the
// parent XML, added to the parent's states as <transition> / <moment> nodes.
//
//   cg_xshlemb parent.xml [-f daughter.xml] [-o out.xml] [-w] [-u] [-ft] [-p]
//              [--system NAME] [--daughter NAME] [--operator NAME]
//
// -f: the daughter system's XML (default: the parent's file); -o: the output
// XML (default: parent.xml itself); -w: Weisskopf units; -u: standard units;
// -ft: log ft; -p: oscillator radial functions positive at infinity.
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-f", "-o", "--system", "--daughter", "--operator"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr,
                 "usage: cg_xshlemb parent.xml [-f daughter.xml] [-o out.xml] [-w] [-u] [-ft] [-p] [--system NAME]"
                 " [--daughter NAME] [--operator NAME]\n");
    return 1;
  }
  const std::string d = a.gets("-f", ""), out = a.gets("-o", ""), ps = a.gets("--system", ""),
                    ds = a.gets("--daughter", ""), op = a.gets("--operator", "");
  const int flags = (a.has("-w") ? CG_EMB_WEISSKOPF : 0) | (a.has("-u") ? CG_EMB_UNITS : 0) |
                    (a.has("-ft") ? CG_EMB_LOGFT : 0) | (a.has("-p") ? CG_EMB_PHASE_INFINITY : 0);
  cli::check(cg_xshlemb(a.pos[0].c_str(), ps.empty() ? nullptr : ps.c_str(), d.empty() ? nullptr : d.c_str(),
                        ds.empty() ? nullptr : ds.c_str(), out.empty() ? nullptr : out.c_str(), flags,
                        op.empty() ? nullptr : op.c_str()),
             "xshlemb");
  return 0;
}
