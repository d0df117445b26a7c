// tests/dropin/driver_main.cpp -- test driver for the GPU drop-in of the
// MCState module: the call sequence of the reference's driver
// (src/Main.cpp:36-189) with a small INPUT reader of its own (the keyword
// rules of src/readInput.cpp:59-257), so that the drop-in can run where the
// reference's own Main.cpp and readInput.cpp are not present.
//
// Built with -DJMM_DRIVER_TEAM the calls are made as the reference's driver
// makes them: inside one OpenMP parallel region, every thread calling fad,
// incrementStep, Step and printG, one thread (single / sections) the
// prints and adjustments, with barriers around Step (src/Main.cpp:50-180).
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "jmmMCState.h"

static MCInput read_input(const char *path) {
  MCInput inp;
  inp.isRestart = false;
  inp.numComputes = 0;
  inp.relaxFlag = 0;
  inp.potCutOff = INFINITY;
  strncpy(inp.ensembleStr, "NPT", 80);
  strncpy(inp.potStr, "LJ", 80);
  FILE *f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "no %s\n", path);
    exit(2);
  }
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    char *tok[8] = {0};
    int nt = 0;
    for (char *t = strtok(line, "[ \t\n]"); t && nt < 8; t = strtok(nullptr, "[ \t\n]")) tok[nt++] = t;
    if (nt == 0) continue;
    const char *k = tok[0];
    const double v = nt > 1 ? strtod(tok[1], nullptr) : 0.0;
    if (!strcmp(k, "RESTART")) inp.isRestart = !(nt > 1 && (!strcmp(tok[1], "FALSE") || !strcmp(tok[1], "False") || !strcmp(tok[1], "false")));
    else if (!strcmp(k, "N")) inp.N = (unsigned long)v;
    else if (!strcmp(k, "P")) inp.P = v;
    else if (!strcmp(k, "L")) inp.L = v;
    else if (!strcmp(k, "T")) inp.T = v;
    else if (!strcmp(k, "NBN")) inp.nbn = (int)v;
    else if (!strcmp(k, "NUMSTEPS")) inp.ns = (unsigned long)v;
    else if (!strcmp(k, "POT")) {
      strncpy(inp.potStr, tok[1], 80);
      inp.potCutOff = nt > 2 ? strtod(tok[2], nullptr) : INFINITY;
    }
    else if (!strcmp(k, "MAXSTEP")) inp.maxStep = v;
    else if (!strcmp(k, "MAXDV")) inp.maxdl = v;
    else if (!strcmp(k, "CPI")) inp.cpi = (unsigned long)v;
    else if (!strcmp(k, "TPI")) inp.tpi = (unsigned long)v;
    else if (!strcmp(k, "GPI")) inp.gpi = (unsigned long)v;
    else if (!strcmp(k, "RHOPI")) inp.rhopi = (unsigned long)v;
    else if (!strcmp(k, "RBW")) inp.rbw = v;
    else if (!strcmp(k, "RHONB")) inp.rhonb = (unsigned long)v;
    else if (!strcmp(k, "GBW")) inp.gbw = v;
    else if (!strcmp(k, "GNB")) inp.gnb = (unsigned long)v;
    else if (!strcmp(k, "GSW")) inp.gsw = v;
    else if (!strcmp(k, "GNS")) inp.gns = (int)v;
    else if (!strcmp(k, "SEED")) inp.seed = (unsigned long)v;
    else if (!strcmp(k, "ENGCHECK")) inp.eci = (unsigned long)v;
    else if (!strcmp(k, "DADJ")) inp.mdai = (unsigned long)v;
    else if (!strcmp(k, "VADJ")) inp.mvai = (unsigned long)v;
    else if (!strcmp(k, "RELAX")) inp.relaxFlag = 1;
    else if (!strcmp(k, "ENSEMBLE")) strncpy(inp.ensembleStr, tok[1], 80);
  }
  fclose(f);
  return inp;
}

#ifndef JMM_DRIVER_TEAM
int main() {
  MCInput inp = read_input("INPUT");
  MCState *mcs = setupMCS(inp);
  if (!mcs) return 1;
  printStep(mcs);
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
  while (incrementStep(mcs)) {
    Step(mcs);
    if (isCoordPrint(mcs)) printCoords(mcs);
    if (isThermoPrint(mcs)) printThermo(mcs);
    if (isRhoPrint(mcs)) printRho(mcs);
    if (isMaxDisAdjust(mcs)) maxDisAdjust(mcs);
    if (isMaxDVAdjust(mcs)) maxDVAdjust(mcs);
    if (isGPrint(mcs)) printG(mcs);
    if ((getStepNum(mcs) % 10000 == 0) && (getStepNum(mcs) < 1E6) && (getRelaxFlag(mcs) > 0))
      relaxVolume(mcs);
  }
  printf("\nPROGRAM COMPLETED SUCCESSFULLY!\n");
  printE(mcs);
  printAcc(mcs);
  freeMCS(mcs);
  return 0;
}
#else
#include <omp.h>

int main() {
  MCInput inp = read_input("INPUT");
  MCState *mcs = setupMCS(inp);
  if (!mcs) return 1;
#pragma omp parallel default(shared)
  {
#pragma omp single
    printStep(mcs);
    unsigned long int nnn = 0;
    double ddd = 0.5;
    fad(mcs, &nnn, &ddd);
    if (getRelaxFlag(mcs) > 0) relaxVolume(mcs);
    if (!getRestartFlag(mcs)) {
#pragma omp sections
      {
#pragma omp section
        printCoords(mcs);
#pragma omp section
        printRho(mcs);
#pragma omp section
        {
          updateThermo(mcs);
          printThermo(mcs);
        }
      }
      printG(mcs);
    }
    while (incrementStep(mcs)) {
#pragma omp barrier
      Step(mcs);
#pragma omp barrier
#pragma omp single
      if (isCoordPrint(mcs)) printCoords(mcs);
#pragma omp single
      if (isThermoPrint(mcs)) printThermo(mcs);
#pragma omp single
      if (isRhoPrint(mcs)) printRho(mcs);
#pragma omp single
      if (isMaxDisAdjust(mcs)) maxDisAdjust(mcs);
#pragma omp single
      if (isMaxDVAdjust(mcs)) maxDVAdjust(mcs);
      if (isGPrint(mcs)) printG(mcs);
      if ((getStepNum(mcs) % 10000 == 0) && (getStepNum(mcs) < 1E6) && (getRelaxFlag(mcs) > 0))
        relaxVolume(mcs);
    }
#pragma omp barrier
  }
  printf("\nPROGRAM COMPLETED SUCCESSFULLY!\n");
  printE(mcs);
  printAcc(mcs);
  freeMCS(mcs);
  return 0;
}
#endif
