// Host-side helpers of the drop-in driver that need no GPU.
//
// pf_ran2 restates the saved-state generator ran_2 of src/ran_2.f90:1-40
// (L'Ecuyer combined generator with a 32-entry Bays-Durham shuffle).  The
// saved Fortran variables (iv, iy, idum2) live in a caller-owned state so that
// several runs can draw independent streams.
#include <cstring>

#include "../../include/pfgpu.h"

namespace {
const int IM1 = 2147483563, IM2 = 2147483399, IMM1 = IM1 - 1;
const int IA1 = 40014, IA2 = 40692, IQ1 = 53668, IQ2 = 52774, IR1 = 12211, IR2 = 3791;
const int NTAB = 32, NDIV = 1 + IMM1 / NTAB;
// am = 1./im1 is evaluated in REAL*4 (src/ran_2.f90:5): both the conversion of
// im1 and the quotient round to single precision before widening.
const double AM = (double)(1.0f / (float)IM1);
const double EPS = 1.2e-7;
const double RNMX = 1.0 - EPS;
}  // namespace

extern "C" {

void pf_ran2_init(pf_ran2_state* st) {
  memset(st, 0, sizeof *st);
  st->idum2 = 123456789;  // data idum2 /123456789/, iv /ntab*0/, iy /0/
}

double pf_ran2(pf_ran2_state* st, int* idum_p) {
  int idum = *idum_p;
  int k, j;
  if (idum <= 0) {
    idum = (-idum > 1) ? -idum : 1;
    st->idum2 = idum;
    for (j = NTAB + 8; j >= 1; --j) {
      k = idum / IQ1;
      idum = IA1 * (idum - k * IQ1) - k * IR1;
      if (idum < 0) idum += IM1;
      if (j <= NTAB) st->iv[j - 1] = idum;
    }
    st->iy = st->iv[0];
  }
  k = idum / IQ1;
  idum = IA1 * (idum - k * IQ1) - k * IR1;
  if (idum < 0) idum += IM1;
  k = st->idum2 / IQ2;
  st->idum2 = IA2 * (st->idum2 - k * IQ2) - k * IR2;
  if (st->idum2 < 0) st->idum2 += IM2;
  j = 1 + st->iy / NDIV;
  st->iy = st->iv[j - 1] - st->idum2;
  st->iv[j - 1] = idum;
  if (st->iy < 1) st->iy += IMM1;
  *idum_p = idum;
  const double v = AM * (double)st->iy;
  return v < RNMX ? v : RNMX;
}

}  // extern "C"
