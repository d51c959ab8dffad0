// Host-side check of vfs::widen (the integer-pipe binary32 -> binary64
// widening the FP64 Krylov kernels apply to FP32 directions) against the
// compiler's conversion.  argv[1] = stride through the 2^32 bit patterns
// (1 = exhaustive); every special class is also checked explicitly.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include "vfs_common.cuh"

static bool same(unsigned u) {
  float f;
  std::memcpy(&f, &u, 4);
  const double a = vfs::widen(f), b = (double)f;
  return std::memcmp(&a, &b, 8) == 0;
}

int main(int argc, char** argv) {
  const unsigned long long stride = argc > 1 ? std::strtoull(argv[1], nullptr, 10) : 1;
  unsigned long long bad = 0, n = 0;
  for (unsigned long long t = 0; t <= 0xffffffffull; t += stride, n++)
    if (!same((unsigned)t)) bad++;
  const unsigned special[] = {0u, 0x80000000u, 1u, 0x80000001u, 0x007fffffu, 0x00400000u, 0x00000100u,
                              0x00800000u, 0x7f7fffffu, 0x7f800000u, 0xff800000u, 0x7fc00000u, 0x7f800001u,
                              0xffbfffffu, 0x3f800000u, 0xbf800000u};
  for (unsigned u : special) {
    n++;
    if (!same(u)) bad++;
  }
  std::printf("checked %llu patterns, %llu mismatches\n", n, bad);
  return bad ? 1 : 0;
}
