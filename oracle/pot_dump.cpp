// oracle/pot_dump.cpp -- TEST INFRASTRUCTURE (the oracle), never shipped.
//
// Calls the reference's own pair functions (src/pot.cpp:19-141, compiled
// unmodified from its own tree by oracle/Makefile) on the separations given
// on standard input and prints phi[0..8] of each as C99 hexadecimal floats,
// so that a test can compare them bit for bit.
//
// Input lines: <potential> <d> <cut-off> <virial 0|1> <L>
//   potential 0 = phiLJcut, 1 = phiLJinfcutoff, 2 = phiHarmoniccut
//   (the jmm_params numbering); params = {virial ? 1 : 0, L}, as the
//   reference's setupMCS passes them.  phiHarmoniccut leaves phi[2..8]
//   unwritten: they are 0 here, and its virial reads L only when
//   params[0] == 1, so it is asked with virial 1 only.
#include <stdio.h>

#include "pot.h"

int main() {
  int pot, virial;
  double d, cut, l;
  while (scanf("%d %lf %lf %d %lf", &pot, &d, &cut, &virial, &l) == 5) {
    double params[3] = {virial ? 1.0 : 0.0, l, cut};
    double phi[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    if (pot == 0)
      phiLJcut(&d, cut, params, phi);
    else if (pot == 1)
      phiLJinfcutoff(&d, cut, params, phi);
    else
      phiHarmoniccut(&d, cut, params, phi);
    for (int k = 0; k < 9; ++k) printf(k ? " %a" : "%a", phi[k]);
    printf("\n");
  }
  return 0;
}
