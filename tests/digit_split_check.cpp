// The digit split of the complex128 split products (zgemm_oz.cu, digits_f64) in its two forms,
// compared bit for bit on the host: the closed form (bytes of V = T + 128 sum 256^j, one
// exact FMA per digit) against the carry loop it replaced.  Integer and IEEE float
// arithmetic only, so the host results are the device's.  Prints the mismatch count per
// digit count and exits non-zero on any mismatch.
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <cmath>
#include <random>
#include <cstdlib>
static float as_f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t as_u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static long long as_ll(double d) { long long b; memcpy(&b, &d, 8); return b; }
template <int S> static long long Tof(double x, int e) {
  const long long bits = as_ll(x);
  const int ex = (int)((bits >> 52) & 0x7FF);
  long long T = 0;
  if (ex != 0) {
    const long long m = (bits & 0xFFFFFFFFFFFFFll) | (1ll << 52);
    const int sh = ex - 1075 + 8 * S - e;
    if (sh >= 0) T = m << sh;
    else if (sh > -63) T = (m + (1ll << (-sh - 1))) >> (-sh);
    if (bits < 0) T = -T;
  }
  return T;
}
template <int S> static void old_d(double x, int e, float* D) {
  long long T = Tof<S>(x, e);
  int d[S];
  for (int s = S - 1; s >= 1; --s) {
    const int lo = (int)((unsigned)T & 255u);
    const int di = ((lo + 128) & 255) - 128;
    d[s] = di;
    T = (T - di) >> 8;
  }
  d[0] = (int)T;
  for (int s = 0; s < S; ++s) {
    const float f = as_f(0x4B400000 + d[s]) - 12582912.0f;
    D[s] = f * as_f((127 - 8 * s) << 23);
  }
}
template <int S> static void new_d(double x, int e, float* D) {
  const long long T = Tof<S>(x, e);
  unsigned long long K = 0;
  for (int j = 0; j < S - 1; ++j) K |= 0x80ull << (8 * j);
  const unsigned long long V = (unsigned long long)T + K;
  for (int j = 0; j < S - 1; ++j) {
    const int s = S - 1 - j;
    const unsigned byte = (unsigned)(V >> (8 * j)) & 255u;
    const float sc = as_f((127 - 8 * s) << 23);
    D[s] = fmaf(as_f(0x4B400000u | byte), sc, -12583040.0f * sc);
  }
  const int top = (int)((long long)V >> (8 * (S - 1)));
  D[0] = as_f(0x4B400000 + top) - 12582912.0f;
}
template <int S> static long long run(std::mt19937_64& g, long long n) {
  long long bad = 0;
  std::uniform_real_distribution<double> u(-1.0, 1.0);
  std::uniform_int_distribution<int> ex(-300, 300);
  for (long long i = 0; i < n; ++i) {
    double x;
    const int mode = i % 5;
    if (mode == 0) x = u(g);
    else if (mode == 1) x = u(g) * std::ldexp(1.0, ex(g));
    else if (mode == 2) x = (double)(long long)(u(g) * 1e6) / 1024.0;
    else if (mode == 3) x = (i & 1 ? -1.0 : 1.0) * std::ldexp(1.0, ex(g));
    else { unsigned long long b = g(); memcpy(&x, &b, 8); if (!std::isfinite(x)) x = 0.0; }
    // e: the exponent bound the prologue gives (|x| <= 2^e), sometimes larger
    int fe; std::frexp(x, &fe);
    const int e = (x == 0.0 ? 0 : fe) + (int)(g() % 3);
    float a[S], b[S];
    old_d<S>(x, e, a); new_d<S>(x, e, b);
    for (int s = 0; s < S; ++s) if (as_u(a[s]) != as_u(b[s])) { ++bad; break; }
  }
  return bad;
}
int main(int argc, char** argv) {
  std::mt19937_64 g(12345);
  const long long n = argc > 1 ? atoll(argv[1]) : 1000000;
  const long long b4 = run<4>(g, n), b6 = run<6>(g, n), b7 = run<7>(g, n);
  printf("S=4 mismatches %lld\nS=6 mismatches %lld\nS=7 mismatches %lld\n", b4, b6, b7);
  return (b4 || b6 || b7) ? 1 : 0;
}
