// oracle/input_dump.cpp -- TEST INFRASTRUCTURE (the oracle), never shipped.
//
// Runs the reference's own INPUT reader (src/readInput.cpp:8-262, compiled
// unmodified from its own tree by oracle/Makefile) on one file and prints
// every field of the struct MCInput it returns (src/jmmMCState.h:50-85), one
// "KEY value" line each, doubles with 17 significant digits.  readInput
// leaves a field uninitialised when its keyword is absent, so a caller
// compares only the fields whose keywords the file names.
//
// Usage: input_dump <INPUT file>
#include <stdio.h>

#include "jmmMCState.h"
#include "readInput.h"

int main(int argc, char **argv) {
  if (argc != 2) {
    fprintf(stderr, "usage: input_dump <INPUT file>\n");
    return 2;
  }
  struct MCInput inp = readInput(argv[1]);
  // readInput prints its own warnings on stdout; a marker separates them
  printf("@@ MCInput\n");
  printf("RESTART %d\n", inp.isRestart ? 1 : 0);
  printf("N %lu\n", inp.N);
  printf("P %.17g\n", inp.P);
  printf("L %.17g\n", inp.L);
  printf("T %.17g\n", inp.T);
  printf("NUMSTEPS %lu\n", inp.ns);
  printf("RELAX %d\n", inp.relaxFlag);
  printf("CPI %lu\n", inp.cpi);
  printf("TPI %lu\n", inp.tpi);
  printf("ENGCHECK %lu\n", inp.eci);
  printf("DADJ %lu\n", inp.mdai);
  printf("VADJ %lu\n", inp.mvai);
  printf("GPI %lu\n", inp.gpi);
  printf("RHOPI %lu\n", inp.rhopi);
  printf("GNB %lu\n", inp.gnb);
  printf("RHONB %lu\n", inp.rhonb);
  printf("SEED %lu\n", inp.seed);
  printf("MAXSTEP %.17g\n", inp.maxStep);
  printf("MAXDV %.17g\n", inp.maxdl);
  printf("CUTOFF %.17g\n", inp.potCutOff);
  printf("POT %.80s\n", inp.potStr);
  printf("ENSEMBLE %.80s\n", inp.ensembleStr);
  printf("RBW %.17g\n", inp.rbw);
  printf("GSW %.17g\n", inp.gsw);
  printf("GBW %.17g\n", inp.gbw);
  printf("GNS %d\n", inp.gns);
  printf("NBN %d\n", inp.nbn);
  // (the argument strings of a COMPUTE line sit in uninitialised storage
  // after its last token, so only the count is printed)
  printf("COMPUTES %d\n", inp.numComputes);
  return 0;
}
