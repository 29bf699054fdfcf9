// The C++ mirror's SaveWavefunction / LoadWavefunction (host only):
//   wavefunction_io save NAME L STRINGS_A STRINGS_B W.bin   -> writes NAME000000
//   wavefunction_io load NAME STRINGS_A STRINGS_B OUT.bin   -> mapped, normalised W
// String files hold one uint64 per line (decimal).
#include <fstream>
#include <iostream>
#include <string>

#include "sbdgb/tpb.hpp"

static std::vector<uint64_t> read_list(const std::string &path) {
  std::ifstream f(path);
  std::vector<uint64_t> v;
  unsigned long long x;
  while (f >> x) v.push_back(x);
  return v;
}

int main(int argc, char **argv) {
  if (argc < 6) return 2;
  const std::string mode = argv[1];
  if (mode == "save") {
    const int L = std::atoi(argv[3]);
    auto a = read_list(argv[4]), b = read_list(argv[5]);
    std::vector<double> W(a.size() * b.size());
    std::ifstream f(argv[6], std::ios::binary);
    f.read((char *)W.data(), (std::streamsize)(sizeof(double) * W.size()));
    sbdgb::SaveWavefunction(argv[2], a, b, L, W);
  } else {
    auto a = read_list(argv[3]), b = read_list(argv[4]);
    std::vector<double> W;
    sbdgb::LoadWavefunction(argv[2], a, b, W);
    std::ofstream f(argv[5], std::ios::binary);
    f.write((const char *)W.data(), (std::streamsize)(sizeof(double) * W.size()));
  }
  return 0;
}
