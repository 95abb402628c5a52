// Caller-side check of the C++ multi-exponentiation drop-in: the reference's call shape
// (test/main.cpp:118, multiexp<FieldT, FieldMul>(v, mul)) on the new element types.
// Usage: multiexp_dropin <field 0|1|2> <n> <a.bin> <b.bin> <out.bin>
// Reads n elements of a and b (raw little-endian limbs), writes two result elements: the reference-shaped
// call (Montgomery product of the stored words) and gsn::multiexp with canonical integers.  Exit 0 on
// success, 1 on error (a size mismatch must throw gsn::Error).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gsn_multiexp.h"

template <class F>
static int run(size_t n, const char* fa, const char* fb, const char* fo) {
  std::vector<F> a(n), b(n);
  FILE* ia = std::fopen(fa, "rb");
  FILE* ib = std::fopen(fb, "rb");
  if (!ia || !ib) return 1;
  if (std::fread(a.data(), sizeof(F), n, ia) != n || std::fread(b.data(), sizeof(F), n, ib) != n) return 1;
  std::fclose(ia);
  std::fclose(ib);
  F mont = multiexp<F, F>(a, b);  // the reference's entry point
  F canon = gsn::multiexp<F>(a, b, GSN_MULTIEXP_CANONICAL);
  FILE* o = std::fopen(fo, "wb");
  if (!o) return 1;
  std::fwrite(&mont, sizeof(F), 1, o);
  std::fwrite(&canon, sizeof(F), 1, o);
  std::fclose(o);
  try {
    std::vector<F> shorter(b.begin(), b.end() - 1);
    multiexp<F, F>(a, shorter);
    return 1;
  } catch (const gsn::Error& e) {
    if (e.code != GSN_ERR_ARG) return 1;
  }
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 6) return 1;
  const int field = std::atoi(argv[1]);
  const size_t n = std::strtoull(argv[2], nullptr, 10);
  try {
    switch (field) {
      case 0: return run<gsn::Fp32>(n, argv[3], argv[4], argv[5]);
      case 1: return run<gsn::FrBLS12_381>(n, argv[3], argv[4], argv[5]);
      case 2: return run<gsn::FrMNT4_753>(n, argv[3], argv[4], argv[5]);
    }
  } catch (const std::exception& e) {
    std::fprintf(stderr, "%s\n", e.what());
  }
  return 1;
}
