// Drop-in for XSHLSF (xmlshell/XSHLSF.cpp:40-222): spectroscopic factors of
// one-particle removal between the <state>s of a parent system and those of a
// daughter system with one particle less (overlaps when the numbers are equal).
//
//   cg_xshlsf parent.xml [-f daughter.xml] [-o out.txt] [-of] [--system NAME] [--daughter NAME]
//
// -f: the daughter system's XML (default: the parent's file); -o: table per
// orbital l; with -of the table per s.p. state (l, 2j, A, SF).
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-f", "-o", "--system", "--daughter"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr,
                 "usage: cg_xshlsf parent.xml [-f daughter.xml] [-o out.txt] [-of] [--system NAME] [--daughter NAME]\n");
    return 1;
  }
  const std::string d = a.gets("-f", ""), out = a.gets("-o", ""), ps = a.gets("--system", ""),
                    ds = a.gets("--daughter", "");
  cli::check(cg_xshlsf(a.pos[0].c_str(), ps.empty() ? nullptr : ps.c_str(), d.empty() ? nullptr : d.c_str(),
                       ds.empty() ? nullptr : ds.c_str(), out.empty() ? nullptr : out.c_str(), a.has("-of") ? 1 : 0),
             "xshlsf");
  return 0;
}
