// oracle/ref_harness.cpp -- TEST INFRASTRUCTURE (the oracle), never shipped.
//
// Builds the reference's own move loop from its own sources, unmodified,
// where they lie (the recipe in oracle/Makefile passes -I to the reference
// tree).  jmmMCState.cpp is compiled into this translation unit so that the
// harness can read the opaque struct MCState (src/jmmMCState.cpp:33-211)
// after every step and log it; the call sequence is the reference driver's
// (src/Main.cpp:36-180): readInput, setupMCS, fad(0, 0.5), the step-0
// prints, then incrementStep/Step/prints/adjusts until NUMSTEPS.
//
// Usage (in a directory holding INPUT):
//   ref_harness <steps.bin> <final.bin>
// steps.bin  : one record per step (step 0 = after the initial fad)
// final.bin  : N, then r[0..N-1], then the 12 thermo accumulators
// RNG draws can be logged separately with JMM_SHIM_LOG=<path>.
#include "jmmMCState.cpp"
#include "readInput.h"

#include <stdint.h>

struct RefStepRecord {
  uint64_t sn;
  uint64_t nm;
  double rn;
  double e, vir, hv, l;
  double e12, e6, vir12, vir6, hv12, hv6;
  uint64_t d_acc0, d_acc1, v_acc0, v_acc1;
};

static void log_step(FILE *f, struct MCState *mcs) {
  RefStepRecord rec;
  rec.sn = mcs->sn;
  rec.nm = mcs->nm;
  rec.rn = mcs->rn;
  rec.e = mcs->E;
  rec.vir = mcs->Vir;
  rec.hv = mcs->HV;
  rec.l = mcs->l;
  rec.e12 = mcs->E12;
  rec.e6 = mcs->E6;
  rec.vir12 = mcs->Vir12;
  rec.vir6 = mcs->Vir6;
  rec.hv12 = mcs->HV12;
  rec.hv6 = mcs->HV6;
  rec.d_acc0 = mcs->dAcc[0];
  rec.d_acc1 = mcs->dAcc[1];
  rec.v_acc0 = mcs->vAcc[0];
  rec.v_acc1 = mcs->vAcc[1];
  fwrite(&rec, sizeof(rec), 1, f);
}

int main(int argc, char **argv) {
  if (argc < 3) {
    fprintf(stderr, "usage: %s <steps.bin> <final.bin>\n", argv[0]);
    return 2;
  }
  FILE *steps = fopen(argv[1], "wb");
  if (!steps) return 3;
  char input_name[] = "INPUT";
  struct MCInput inp = readInput(input_name);
  struct MCState *mcs = setupMCS(inp);
  if (!mcs) return 4;

  unsigned long int nnn = 0;
  double ddd = 0.5;
  fad(mcs, &nnn, &ddd);
  if (getRelaxFlag(mcs) > 0) relaxVolume(mcs);
  if (!getRestartFlag(mcs)) {
    printCoords(mcs);
    printRho(mcs);
    updateThermo(mcs);
    printThermo(mcs);
    printG(mcs);
  }
  log_step(steps, mcs);

  while (incrementStep(mcs)) {
    Step(mcs);
    if (isCoordPrint(mcs)) printCoords(mcs);
    if (isThermoPrint(mcs)) printThermo(mcs);
    if (isRhoPrint(mcs)) printRho(mcs);
    if (isMaxDisAdjust(mcs)) maxDisAdjust(mcs);
    if (isMaxDVAdjust(mcs)) maxDVAdjust(mcs);
    if (isGPrint(mcs)) printG(mcs);
    if ((getStepNum(mcs) % 10000 == 0) && (getStepNum(mcs) < 1E6) &&
        (getRelaxFlag(mcs) > 0))
      relaxVolume(mcs);
    log_step(steps, mcs);
  }
  fclose(steps);

  FILE *fin = fopen(argv[2], "wb");
  if (fin) {
    uint64_t n = mcs->N;
    fwrite(&n, sizeof(n), 1, fin);
    fwrite(mcs->r, sizeof(double), mcs->N, fin);
    double accs[12] = {mcs->rhoSysA, mcs->rhoSysSA, mcs->lA,  mcs->lSA,
                       mcs->EA,      mcs->ESA,      mcs->lEA, mcs->VirA,
                       mcs->VirSA,   mcs->EVirA,    mcs->HVA, mcs->HVSA};
    fwrite(accs, sizeof(double), 12, fin);
    fclose(fin);
  }
  printE(mcs);
  printAcc(mcs);
  return 0;
}
