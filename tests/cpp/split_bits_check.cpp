// Reads FP64 values (binary, native order) and writes, per value, the FP32
// bits, the BF16 bits and whether split_bits handled it (uint32, uint32,
// uint32), for the host check of the integer FP64 -> FP32 + BF16 split.
#include <cstdio>
#include <cstring>
#include <vector>

#include "split_bits.h"

int main(int argc, char** argv) {
  if (argc != 3) return 2;
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 3;
  std::vector<double> x;
  double v;
  while (std::fread(&v, sizeof v, 1, f) == 1) x.push_back(v);
  std::fclose(f);
  FILE* g = std::fopen(argv[2], "wb");
  if (!g) return 4;
  for (double d : x) {
    uint64_t b;
    std::memcpy(&b, &d, sizeof b);
    uint32_t hb = 0;
    uint16_t lb = 0;
    const bool ok = fvg::split_bits(b, &hb, &lb);
    const uint32_t o[3] = {hb, lb, ok ? 1u : 0u};
    std::fwrite(o, sizeof o, 1, g);
  }
  std::fclose(g);
  return 0;
}
