// Host-side check of the in-register DFTs and the four-step line plans of
// pf_fft.cuh (compiled by tests/test_fft_host.py; no GPU needed).  For every
// radix and every line length it prints the largest error against a plain
// FP64 DFT, relative to the largest output magnitude:
//   dft <R> <forward err> <inverse err>
//   line <L> <forward err>
//   xline <L> <forward err>   (the x pass's own factorization, where it differs)
// The line transform runs pass A (DFT_N2 of the columns n1, twiddles
// W_L^(n1 k2)) then pass B (DFT_N1 of the rows k2), exactly as the shared-
// memory passes do, and reads frequency k at position pos_of_freq(k).
#include <cmath>
#include <complex>
#include <cstdio>
#include <random>
#include <vector>

#include "pf_fft.cuh"

using namespace pf;
using cd = std::complex<double>;

static std::vector<cd> dft_ref(const std::vector<cd>& x, int sign) {
  const int n = (int)x.size();
  std::vector<cd> X(n);
  for (int k = 0; k < n; ++k) {
    cd s = 0;
    for (int j = 0; j < n; ++j) {
      const double a = sign * 2.0 * M_PI * (double)((long long)j * k % n) / n;
      s += x[j] * cd(std::cos(a), std::sin(a));
    }
    X[k] = s;
  }
  return X;
}

static double rel_err(const std::vector<cd>& got, const std::vector<cd>& ref) {
  double e = 0, m = 0;
  for (size_t i = 0; i < ref.size(); ++i) {
    e = std::max(e, std::abs(got[i] - ref[i]));
    m = std::max(m, std::abs(ref[i]));
  }
  return e / std::max(m, 1e-300);
}

template <int R>
static void check_dft(std::mt19937& g) {
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  float2 v[R], w[R];
  std::vector<cd> x(R);
  for (int i = 0; i < R; ++i) {
    v[i] = make_float2(u(g), u(g));
    w[i] = v[i];
    x[i] = cd(v[i].x, v[i].y);
  }
  Dft<R>::fwd(v);
  dft_inv<R>(w);
  std::vector<cd> a(R), b(R);
  for (int i = 0; i < R; ++i) {
    a[i] = cd(v[i].x, v[i].y);
    b[i] = cd(w[i].x, w[i].y);
  }
  printf("dft %d %.3e %.3e\n", R, rel_err(a, dft_ref(x, -1)), rel_err(b, dft_ref(x, +1)));
}

// LN: the line type (its length, runs N1 and strides N2); tag: "line" for a
// plan's factorization, "xline" for the x pass's own factorization.
template <int L, class LN = Line<L>>
static void check_line(std::mt19937& g, const char* tag = "line") {
  constexpr int N1 = LN::N1, N2 = LN::N2;
  std::uniform_real_distribution<float> u(-1.f, 1.f);
  std::vector<float2> buf(L), tw(L);
  std::vector<cd> x(L);
  for (int j = 0; j < L; ++j) {
    buf[j] = make_float2(u(g), u(g));
    x[j] = cd(buf[j].x, buf[j].y);
    const double a = 2.0 * M_PI * j / L;
    tw[j] = make_float2((float)std::cos(a), (float)-std::sin(a));
  }
  for (int n1 = 0; n1 < N1; ++n1) {  // pass A
    float2 v[N2];
    for (int n2 = 0; n2 < N2; ++n2) v[n2] = buf[n1 + N1 * n2];
    Dft<N2>::fwd(v);
    for (int k2 = 1; k2 < N2; ++k2) v[k2] = cmul(v[k2], tw[n1 * k2]);
    for (int k2 = 0; k2 < N2; ++k2) buf[n1 + N1 * k2] = v[k2];
  }
  for (int k2 = 0; k2 < N2; ++k2) {  // pass B
    float2 w[N1];
    for (int n1 = 0; n1 < N1; ++n1) w[n1] = buf[n1 + N1 * k2];
    Dft<N1>::fwd(w);
    for (int k1 = 0; k1 < N1; ++k1) buf[k1 + N1 * k2] = w[k1];
  }
  std::vector<cd> got(L);
  for (int k = 0; k < L; ++k) {
    const float2 c = buf[LN::pos_of_freq(k)];
    got[k] = cd(c.x, c.y);
  }
  printf("%s %d %.3e\n", tag, L, rel_err(got, dft_ref(x, -1)));
}

int main() {
  std::mt19937 g(12345);
  check_dft<2>(g); check_dft<3>(g); check_dft<4>(g); check_dft<5>(g); check_dft<6>(g); check_dft<8>(g);
  check_dft<10>(g); check_dft<12>(g); check_dft<16>(g); check_dft<17>(g); check_dft<20>(g);
  check_line<4>(g); check_line<8>(g); check_line<12>(g); check_line<16>(g); check_line<24>(g);
  check_line<32>(g); check_line<40>(g); check_line<48>(g); check_line<51>(g); check_line<64>(g); check_line<80>(g);
  check_line<96>(g); check_line<100>(g); check_line<102>(g); check_line<128>(g); check_line<160>(g); check_line<192>(g);
  check_line<200>(g); check_line<256>(g);
  // the x pass's lines of 128 complex points (Nx = 256) as 8 x 16
  check_line<128, Line<128, 8, 16>>(g, "xline");
  return 0;
}
