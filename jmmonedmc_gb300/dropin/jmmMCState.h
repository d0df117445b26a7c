// jmmMCState.h -- the MCState API of jmmOneDMC's move loop, as the drop-in
// in this directory implements it on libjmmgpu.so.
//
// The declarations must be those of the reference's own header
// (src/jmmMCState.h:6-48, struct MCInput :50-85): the reference's driver
// (src/Main.cpp) and INPUT reader (src/readInput.cpp) are compiled against
// them unchanged, so every signature and the field order and types of
// MCInput are kept.  Either this header or the reference's may be on the
// include path; they describe the same interface.
#ifndef JMM_DROPIN_MCSTATE_H
#define JMM_DROPIN_MCSTATE_H

#include <stdbool.h>

#include <vector>

extern double lRat1, lRat3, lRat6, lRat7, lRat12, lRat13;

struct MCState;
struct MCState *setupMCS(struct MCInput inp);
void freeMCS(struct MCState *);
void printStep(struct MCState *);
int printMCP(struct MCState *mcs1);
int printThermo(struct MCState *mcs);
int printCoords(struct MCState *mcs);
int printRho(struct MCState *mcs);
int printG(struct MCState *mcs);
int fgrho(struct MCState *mcs);
int ugrho(struct MCState *mcs);
int qagrho(struct MCState *mcs);
int NPTtrial(struct MCState *mcs);
int fad(struct MCState *, unsigned long int *, double *);
int qad(struct MCState *mcs, unsigned long int *nm, double *d);
int qad2(struct MCState *mcs, unsigned long int *nm, double *d);
int fav(struct MCState *mcs);
int qav(struct MCState *mcs);
int qavLJ(struct MCState *mcs);
int qavHarmonic(struct MCState *mcs);
unsigned long int incrementStep(struct MCState *mcs);
int Step(struct MCState *mcs);
int isCoordPrint(struct MCState *mcs);
int isThermoPrint(struct MCState *mcs);
int isRhoPrint(struct MCState *mcs);
int isGPrint(struct MCState *mcs);
int isECheck(struct MCState *mcs);
int isMaxDisAdjust(struct MCState *mcs);
int isMaxDVAdjust(struct MCState *mcs);
int updateThermo(struct MCState *mcs);
int ECheck(struct MCState *mcs);
int MaxDisAdjust(struct MCState *mcs);
int MaxDVAdjust(struct MCState *mcs);
int relaxVolume(struct MCState *mcs);
unsigned long int getStepNum(struct MCState *mcs);
double calculateEnergyOfTrialVolumeChange(struct MCState *mcs, double dl);
int moveVolume(struct MCState *mcs, double l);
int getRelaxFlag(struct MCState *mcs);
bool getRestartFlag(struct MCState *mcs);
int maxDisAdjust(struct MCState *mcs);
int maxDVAdjust(struct MCState *mcs);
int printE(struct MCState *mcs);
int printAcc(struct MCState *mcs);

// The INPUT keywords, filled by readInput (field order and types are the
// reference's: readInput.cpp writes them by name into this layout).
struct MCInput {
  bool isRestart;
  unsigned long int N;
  unsigned long int numTrialTypes;
  double P;
  double L;
  double T;
  unsigned long int ns;
  int relaxFlag;
  unsigned long int cpi;
  unsigned long int tpi;
  unsigned long int eci;
  unsigned long int mdai;
  unsigned long int mvai;
  unsigned long int gpi;
  unsigned long int rhopi;
  unsigned long int gnb;
  unsigned long int rhonb;
  unsigned long int seed;
  double maxStep;
  double maxdl;
  double potCutOff;
  char potStr[80];
  char ensembleStr[80];
  double rbw;
  double gsw;
  double gbw;
  int gns;
  int nbn;

  int numComputes;
  std::vector<char **> computeStrs;
};

#endif
