// jmmMCState.cpp -- drop-in replacement of the reference's MCState module
// (src/jmmMCState.cpp) on libjmmgpu.so.
//
// The reference's driver (src/Main.cpp) and INPUT reader (src/readInput.cpp)
// link against this file unchanged: every function of src/jmmMCState.h that
// the reference defines is defined here with the same signature.  The move
// loop runs on the GPU through the C ABI of include/jmm_gpu.h (the plain FP64
// form, which reproduces the reference's trajectory step for step); this file
// keeps the host-side parts: parameters, step counting, the print cadence and
// the output files config.dat.mcs, thermo.dat.mcs, rho.dat.mcs and
// g<k>.dat.mcs in the reference's formats (src/jmmMCState.cpp:1007-1061,
// :1896-1937); the histogram counts themselves are kept on the GPU by the
// move loop (jmm_plain_histograms).
//
// Step() only counts: the counted steps run on the GPU in one launch when
// the driver next needs the chain's state (a print, an adjustment, the
// energy check's message, the end).  The reference's driver calls fad,
// incrementStep, Step and the direct moves from every thread of an OpenMP
// team and the rest from one thread; here the former run once per team
// (omp single, the value broadcast), the latter under a critical section.
//
// fgrho, ugrho and qagrho are run by the GPU move loop where the reference's
// moves call them; called directly they do nothing.  On a restart the
// histogram files keep their lines up to the restart step and are cut there
// (the reference overwrites in place).
#include "jmmMCState.h"

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "jmm_gpu.h"

double lRat1, lRat3, lRat6, lRat7, lRat12, lRat13;

struct MCState {
  jmm_plain *h;
  jmm_params prm;
  bool isRestart;
  unsigned long int N;
  unsigned long int sn;        // host step number (incrementStep)
  unsigned long int dev_sn;    // step number the GPU has reached
  unsigned long int numSteps;
  int relaxFlag;
  unsigned long int cpi, tpi, eci, mdai, mvai, gpi, rhopi, gnb, rhonb, seed;
  unsigned long int sltp, slcp;
  double maxStep, maxdl;
  double rn;                   // trial uniform handed to a direct qav/fav call
  int gns;
  char potStr[20];
  char ensembleStr[80];
  FILE *cf, *tf, *rhof;
  std::vector<FILE *> gf;
  unsigned long int slrho, slg;  // steps of the last rho / g prints
  double rbw, gsw, gbw;
};

namespace {

void report(int rc, const char *what) {
  if (rc != JMM_OK) {
    fprintf(stderr, "jmmMCState (GPU): %s failed: %s\n", what, jmm_last_error());
    exit(1);
  }
}

jmm_state state_of(MCState *mcs) {
  jmm_state st;
  report(jmm_plain_get_state(mcs->h, &st), "jmm_plain_get_state");
  return st;
}

// The energy check's message of src/jmmMCState.cpp:1998-2090.
void echeck_message(MCState *mcs, const jmm_state &st, bool reset) {
  if (reset) {
    fprintf(stdout,
            "\n### !!! $$$ Energy discrepancy!!! ######### !!!!!!!!!!! $$$$$$$$$$ !!!!!!!!\n"
            "E = %.8G, ETest = %.8G, Resetting results to that of full calculation (E = %.8G)\n\n",
            st.echeck_e_before, st.echeck_e, st.echeck_e);
  } else {
    fprintf(stdout, "####### Energy was just verified ########  E = %.8G ######## ETest = %.8G #######\n",
            st.echeck_e_before, st.echeck_e);
  }
}

// Run the steps counted since the last flush, stopping at every energy-check
// step to print its message.
void flush(MCState *mcs) {
  while (mcs->dev_sn < mcs->sn) {
    unsigned long int chunk = mcs->sn - mcs->dev_sn;
    if (mcs->eci) {
      const unsigned long int to_check = mcs->eci - mcs->dev_sn % mcs->eci;
      if (to_check < chunk) chunk = to_check;
    }
    const jmm_state before = mcs->eci ? state_of(mcs) : jmm_state();
    report(jmm_plain_steps(mcs->h, chunk, nullptr, nullptr), "jmm_plain_steps");
    mcs->dev_sn += chunk;
    if (mcs->eci && mcs->dev_sn % mcs->eci == 0) {
      const jmm_state st = state_of(mcs);
      echeck_message(mcs, st, st.echeck_resets > before.echeck_resets);
    }
  }
  fflush(stdout);
}

// Last complete frame of config.dat.mcs: N, "Step no.: S  Box length: L",
// then N lines "i 0.0 0.0 x" (the format of printCoords).  Truncates the
// file after that frame; returns false when none is complete.
bool read_last_frame(unsigned long int n, std::vector<double> *r, unsigned long int *sn,
                     double *l) {
  FILE *f = fopen("config.dat.mcs", "r");
  if (!f) return false;
  std::vector<std::string> lines;
  char buf[20000];
  while (fgets(buf, sizeof(buf), f)) lines.push_back(buf);
  fclose(f);
  bool found = false;
  size_t end = 0;
  for (size_t k = 0; k + 1 < lines.size(); ++k) {
    unsigned long int npexp = 0, s = 0;
    double box = 0;
    if (sscanf(lines[k].c_str(), "%lu", &npexp) != 1) continue;
    if (sscanf(lines[k + 1].c_str(), "Step no.: %lu Box length: %lf", &s, &box) != 2) continue;
    if (npexp != n) {
      fprintf(stdout, "ERROR: Number of particles in config.mcs.dat (%lu) is incompatible with "
                      "number of particles in INPUT (%lu).\n", npexp, n);
      exit(1);
    }
    if (k + 2 + n > lines.size()) break;
    std::vector<double> x(n);
    bool ok = true;
    for (unsigned long int i = 0; i < n && ok; ++i) {
      unsigned int pn;
      double a, b, z;
      ok = sscanf(lines[k + 2 + i].c_str(), "%u %lg %lg %lg", &pn, &a, &b, &z) == 4;
      x[i] = z;
    }
    if (!ok) break;
    *r = x;
    *sn = s;
    *l = box;
    found = true;
    end = k + 2 + n;
    k = end - 1;
  }
  if (found) {
    f = fopen("config.dat.mcs", "w");
    for (size_t k = 0; k < end; ++k) fputs(lines[k].c_str(), f);
    fclose(f);
  }
  return found;
}

// Keeps the lines of `name` whose step is <= `sn` (and the header line when
// `header`), cuts the rest, and returns the last kept step.
unsigned long int rewind_file(const char *name, unsigned long int sn, bool header) {
  FILE *f = fopen(name, "r");
  std::vector<std::string> keep;
  unsigned long int last = 0;
  if (f) {
    std::vector<char> buf(1 << 20);
    bool first = true;
    while (fgets(buf.data(), (int)buf.size(), f)) {
      unsigned long int s;
      if (first && header) {
        keep.push_back(buf.data());
      } else if (sscanf(buf.data(), "%lu", &s) == 1 && s <= sn) {
        keep.push_back(buf.data());
        last = s;
      }
      first = false;
    }
    fclose(f);
  }
  f = fopen(name, "w");
  for (const auto &line : keep) fputs(line.c_str(), f);
  fclose(f);
  return last;
}

void rewind_thermo(unsigned long int sn) { rewind_file("thermo.dat.mcs", sn, true); }

}  // namespace

int printMCP(struct MCState *mcs) {
  if (mcs->isRestart) printf("*** THIS IS A RESTART RUN ***\n");
  printf("Printing Monte Carlo parameters...\n");
  printf("Ensemble: %s\n", mcs->ensembleStr);
  if (mcs->prm.ensemble == JMM_NPT)
    printf("N: %lu\nP: %.5G\nT: %.5G\n", mcs->N, mcs->prm.p, mcs->prm.t);
  else
    printf("N: %lu\nL: %.5G\nT: %.5G\n", mcs->N, mcs->prm.l, mcs->prm.t);
  printf("Potential: %s\n", mcs->potStr);
  printf("Potential cut-off: %.5G\n", mcs->prm.cutoff);
  printf("numSteps: %lu\nmaxStep: %.5G\nmax vol change: %.5G\n", mcs->numSteps, mcs->maxStep,
         mcs->maxdl);
  printf("Seed: %lu\n", mcs->seed);
  printf("Move loop: libjmmgpu.so (GB300, plain FP64 form)\n\n");
  fflush(stdout);
  return 0;
}

struct MCState *setupMCS(struct MCInput inp) {
  MCState *mcs = new MCState();
  snprintf(mcs->potStr, sizeof(mcs->potStr), "%.19s", inp.potStr);
  snprintf(mcs->ensembleStr, sizeof(mcs->ensembleStr), "%.79s", inp.ensembleStr);
  jmm_params &p = mcs->prm;
  memset(&p, 0, sizeof(p));
  if (strncmp(inp.potStr, "LJ", 10) == 0) {
    p.potential = JMM_POT_LJ;
    p.cutoff = INFINITY;
  } else if (strncmp(inp.potStr, "LJcut", 10) == 0) {
    p.potential = JMM_POT_LJCUT;
    p.cutoff = inp.potCutOff;
  } else if (strncmp(inp.potStr, "HARMONIC", 10) == 0) {
    p.potential = JMM_POT_HARMONIC;
    p.cutoff = inp.potCutOff;
  } else {
    printf("FATAL ERROR: Unknown potential.\nABORTING SIMULATION\n\n");
    delete mcs;
    return nullptr;
  }
  if (strncmp(inp.ensembleStr, "NPT", 80) == 0) {
    printf("ENSEMBLE = NPT\n");
    p.ensemble = JMM_NPT;
    mcs->relaxFlag = inp.relaxFlag;
  } else if (strncmp(inp.ensembleStr, "NLT", 80) == 0) {
    printf("ENSEMBLE = NLT\n");
    p.ensemble = JMM_NLT;
    if (inp.relaxFlag)
      printf("This is an NLT ensemble simulation. Ignoring requested volume relaxation.\n");
    mcs->relaxFlag = 0;
  } else {
    printf("FATAL ERROR: Unknown ensemble.\nABORTING SIMULATION\n\n");
    delete mcs;
    return nullptr;
  }
  p.n = inp.N;
  p.p = inp.P;
  p.l = inp.L;
  p.t = inp.T;
  p.nbn = inp.nbn;
  p.max_step = inp.maxStep;
  p.max_dl = inp.maxdl;
  p.seed = inp.seed;
  p.eci = inp.eci;
  mcs->isRestart = inp.isRestart;
  mcs->N = inp.N;
  mcs->numSteps = inp.ns;
  mcs->cpi = inp.cpi;
  mcs->tpi = inp.tpi;
  mcs->eci = inp.eci;
  mcs->mdai = inp.mdai;
  mcs->mvai = inp.mvai;
  mcs->gpi = inp.gpi;
  mcs->rhopi = inp.rhopi;
  mcs->gnb = inp.gnb;
  mcs->rhonb = inp.rhonb;
  mcs->gns = inp.gns;
  mcs->seed = inp.seed;
  mcs->maxStep = inp.maxStep;
  mcs->maxdl = inp.maxdl;
  mcs->rbw = inp.rbw;
  mcs->gsw = inp.gsw;
  mcs->gbw = inp.gbw;
  mcs->rn = 0.5;
  printMCP(mcs);
  if (jmm_plain_create(&p, &mcs->h) != JMM_OK) {
    printf("FATAL ERROR: %s\nABORTING SIMULATION\n\n", jmm_last_error());
    delete mcs;
    return nullptr;
  }
  if (!mcs->isRestart) {
    mcs->cf = fopen("config.dat.mcs", "w");
    mcs->tf = fopen("thermo.dat.mcs", "w");
    mcs->rhof = fopen("rho.dat.mcs", "w");
    for (int k = 0; k < mcs->gns; ++k) {
      char name[64];
      snprintf(name, sizeof(name), "g%d.dat.mcs", k);
      mcs->gf.push_back(fopen(name, "w"));
    }
    mcs->sn = 0;
    mcs->dev_sn = 0;
    mcs->slcp = (unsigned long int)-1;
    mcs->sltp = (unsigned long int)-1;
    mcs->slrho = (unsigned long int)-1;
    mcs->slg = (unsigned long int)-1;
    fprintf(mcs->tf,
            "Step    Econf           Econf2          L       L2      LEconf          rho"
            "             rho2            Virial         Virial2         EconfVir        HV"
            "              HV2 \n");
  } else {
    std::vector<double> r;
    unsigned long int sn = 0;
    double l = 0;
    printf("Opening file %s\n", "config.dat.mcs");
    if (!read_last_frame(mcs->N, &r, &sn, &l)) {
      printf("FATAL ERROR: no complete configuration in config.dat.mcs\n");
      jmm_plain_destroy(mcs->h);
      delete mcs;
      return nullptr;
    }
    printf("Complete configuration found for step number %lu\n", sn);
    printf("Box length: %.8g\n", l);
    report(jmm_plain_set_config(mcs->h, r.data(), mcs->N, l, sn), "jmm_plain_set_config");
    printf("Opening file %s\n", "rho.dat.mcs");
    const unsigned long int lastrho = rewind_file("rho.dat.mcs", sn, false);
    printf("Last rho time point <= last complete config time point: %lu\n"
           "  Overwriting density data beyond this point.\n", lastrho);
    unsigned long int lastgmin = sn;
    for (int k = 0; k < mcs->gns; ++k) {
      char name[64];
      snprintf(name, sizeof(name), "g%d.dat.mcs", k);
      printf("Opening file %s\n", name);
      const unsigned long int lastg = rewind_file(name, sn, false);
      printf("Last g[%d] time point <= last complete config time point: %lu\n", k, lastg);
      if (lastg < lastgmin) lastgmin = lastg;
      mcs->gf.push_back(fopen(name, "a"));
    }
    printf("Least compatible g time point: %lu\n"
           "  Overwriting g(r) data beyond this point.\n", lastgmin);
    rewind_thermo(sn);
    mcs->cf = fopen("config.dat.mcs", "a");
    mcs->tf = fopen("thermo.dat.mcs", "a");
    mcs->rhof = fopen("rho.dat.mcs", "a");
    mcs->sn = sn;
    mcs->dev_sn = sn;
    mcs->slcp = sn;
    mcs->sltp = sn;
    mcs->slrho = sn;
    mcs->slg = sn;
  }
  // the density and g(x) counts of the starting configuration, accumulated
  // once (setupMCS, src/jmmMCState.cpp:773-776)
  if (jmm_plain_histograms(mcs->h, mcs->rhonb, mcs->rbw, mcs->gns, mcs->gsw, mcs->gnb,
                           mcs->gbw) != JMM_OK) {
    printf("FATAL ERROR: %s\nABORTING SIMULATION\n\n", jmm_last_error());
    freeMCS(mcs);
    return nullptr;
  }
  fflush(mcs->cf);
  fflush(mcs->tf);
  fflush(stdout);
  return mcs;
}

void freeMCS(struct MCState *mcs) {
  if (!mcs) return;
  jmm_plain_destroy(mcs->h);
  if (mcs->cf) fclose(mcs->cf);
  if (mcs->tf) fclose(mcs->tf);
  if (mcs->rhof) fclose(mcs->rhof);
  for (FILE *f : mcs->gf)
    if (f) fclose(f);
  delete mcs;
}

void printStep(struct MCState *mcs) {
  printf("Step: %lu...\n", mcs->sn);
  fflush(stdout);
}

int fad(struct MCState *mcs, unsigned long int *nm, double *d) {
  int rc = 0;
#pragma omp single copyprivate(rc)
  {
    flush(mcs);
    if (!nm || !d) {
      fprintf(stderr, "jmmMCState (GPU): fad needs an explicit particle and uniform\n");
      rc = -1;
    } else {
      report(jmm_plain_fad(mcs->h, *nm, *d), "jmm_plain_fad");
    }
  }
  return rc;
}

static int one_move(struct MCState *mcs, int32_t kind, unsigned long int nm, double rn) {
  flush(mcs);
  report(jmm_plain_move(mcs->h, kind, nm, rn, nullptr), "jmm_plain_move");
  return 0;
}

int qad(struct MCState *mcs, unsigned long int *nm, double *d) { return qad2(mcs, nm, d); }

int qad2(struct MCState *mcs, unsigned long int *nm, double *d) {
  int rc = 0;
#pragma omp single copyprivate(rc)
  {
    if (!nm || !d) {
      fprintf(stderr, "jmmMCState (GPU): qad2 needs an explicit particle and uniform\n");
      rc = -1;
    } else {
      rc = one_move(mcs, JMM_KIND_DISPLACEMENT, *nm, *d);
    }
  }
  return rc;
}

int qav(struct MCState *mcs) {
  int rc = 0;
#pragma omp single copyprivate(rc)
  rc = one_move(mcs, JMM_KIND_VOLUME, 0, mcs->rn);
  return rc;
}

int fav(struct MCState *mcs) { return qav(mcs); }
int qavLJ(struct MCState *mcs) { return qav(mcs); }

// The barrier (src/jmmMCState.cpp:1742) keeps the step number unchanged until
// every thread of the team has finished the previous step's print tests
// (the driver evaluates isGPrint from all threads outside any single); without
// it a fast thread's increment sends a slow one into a different construct.
unsigned long int incrementStep(struct MCState *mcs) {
  unsigned long int out = 0;
#pragma omp barrier
#pragma omp single copyprivate(out)
  {
    if (mcs->sn != mcs->numSteps) {
      mcs->sn++;
      if (mcs->sn % 10000 == 0) printStep(mcs);
      out = mcs->sn;
    }
  }
  return out;
}

// The step itself runs later, in the launch that flush() makes.
int Step(struct MCState *mcs) {
  (void)mcs;
  return 0;
}

int isCoordPrint(struct MCState *mcs) { return mcs->sn % mcs->cpi == 0; }
int isThermoPrint(struct MCState *mcs) { return mcs->sn % mcs->tpi == 0; }
int isRhoPrint(struct MCState *mcs) { return mcs->sn % mcs->rhopi == 0; }
int isGPrint(struct MCState *mcs) { return mcs->sn % mcs->gpi == 0; }
int isECheck(struct MCState *mcs) { return mcs->eci && mcs->sn % mcs->eci == 0; }
int isMaxDisAdjust(struct MCState *mcs) { return mcs->sn % mcs->mdai == 0; }
int isMaxDVAdjust(struct MCState *mcs) { return mcs->sn % mcs->mvai == 0; }

int updateThermo(struct MCState *mcs) {
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    report(jmm_plain_update_thermo(mcs->h), "jmm_plain_update_thermo");
  }
  return 0;
}

int printThermo(struct MCState *mcs) {
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    const jmm_state st = state_of(mcs);
    const unsigned long int ss = mcs->sn - mcs->sltp;
    const double *a = st.thermo;
    fprintf(mcs->tf, "%lu\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\t%.8G\n",
            mcs->sn, a[4] / ss, a[5] / ss, a[2] / ss, a[3] / ss, a[6] / ss, a[0] / ss, a[1] / ss,
            a[7] / ss, a[8] / ss, a[9] / ss, a[10] / ss, a[11] / ss);
    fflush(mcs->tf);
    printf("%lu  %.8G  %.8G  %.8G  %.8G\n", mcs->sn, st.tot[JMM_Q_E], st.l, st.tot[JMM_Q_VIR],
           st.tot[JMM_Q_HV]);
    fflush(stdout);
    report(jmm_plain_reset_thermo(mcs->h), "jmm_plain_reset_thermo");
    mcs->sltp = mcs->sn;
  }
  return 0;
}

int printCoords(struct MCState *mcs) {
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    const jmm_state st = state_of(mcs);
    std::vector<double> r(mcs->N);
    report(jmm_plain_get_positions(mcs->h, r.data(), mcs->N), "jmm_plain_get_positions");
    fprintf(mcs->cf, "%lu\nStep no.: %lu  Box length: %.5f\n", mcs->N, mcs->sn, st.l);
    for (unsigned long int i = 0; i < mcs->N; ++i)
      fprintf(mcs->cf, "%lu  0.0  0.0  %.8G\n", i + 1, r[i]);
    fflush(mcs->cf);
    mcs->slcp = mcs->sn;
  }
  return 0;
}

// printRho (src/jmmMCState.cpp:1021-1037): the density sums since the last
// print, divided by the steps since then and the bin width.
int printRho(struct MCState *mcs) {
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    std::vector<int32_t> acc(mcs->rhonb);
    report(jmm_plain_take_rho(mcs->h, acc.data(), mcs->rhonb), "jmm_plain_take_rho");
    const unsigned long int ns = mcs->sn - mcs->slrho;
    fprintf(mcs->rhof, "%lu", mcs->sn);
    for (unsigned long int rb = 0; rb < mcs->rhonb; ++rb)
      fprintf(mcs->rhof, " %.8G", (double)acc[rb] / ns / mcs->rbw);
    fprintf(mcs->rhof, "\n");
    fflush(mcs->rhof);
    mcs->slrho = mcs->sn;
  }
  return 0;
}

// printG (src/jmmMCState.cpp:1042-1061), which the driver calls from every
// thread of its team: one line per slice file.
int printG(struct MCState *mcs) {
#pragma omp single
  {
#pragma omp critical(jmm_dropin)
    {
      flush(mcs);
      const unsigned long int nbin = (unsigned long int)mcs->gns * mcs->gnb;
      std::vector<int32_t> acc(nbin);
      report(jmm_plain_take_g(mcs->h, acc.data(), nbin), "jmm_plain_take_g");
      const unsigned long int ns = mcs->sn - mcs->slg;
      for (int gs = 0; gs < mcs->gns; ++gs) {
        fprintf(mcs->gf[gs], "%lu", mcs->sn);
        for (unsigned long int gb = 0; gb < mcs->gnb; ++gb)
          fprintf(mcs->gf[gs], " %.8G", (double)acc[gs * mcs->gnb + gb] / ns / mcs->gsw / mcs->gbw);
        fprintf(mcs->gf[gs], "\n");
        fflush(mcs->gf[gs]);
      }
      mcs->slg = mcs->sn;
    }
  }
  return 0;
}

// The histogram updates run inside the GPU move loop where the reference's
// moves call them (qad2, qavLJ) and at set-up; a direct call has nothing to do.
int fgrho(struct MCState *mcs) {
  (void)mcs;
  return 0;
}
int ugrho(struct MCState *mcs) {
  (void)mcs;
  return 0;
}
int qagrho(struct MCState *mcs) {
  (void)mcs;
  return 0;
}

int ECheck(struct MCState *mcs) {
  int32_t reset = 0;
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    double e_test = 0;
    report(jmm_plain_echeck(mcs->h, &e_test, &reset), "jmm_plain_echeck");
    echeck_message(mcs, state_of(mcs), reset != 0);
  }
  return reset;
}

// maxDisAdjust (src/jmmMCState.cpp:2100-2116): Swendsen's rescaling of the
// maximum displacement toward 50 % acceptance from the cumulative counts.
int maxDisAdjust(struct MCState *mcs) {
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    const jmm_state st = state_of(mcs);
    const double ideal = 0.5;
    const double actual = (double)st.d_acc[0] / (st.d_acc[0] + st.d_acc[1]);
    double ms = mcs->maxStep * log(0.672924 * ideal + 0.0644284) /
                log(0.672924 * (actual + 0.0644284));
    if (ms < 0.002)
      ms = 0.002;
    else if (ms > 0.5)
      ms = 0.5;
    mcs->maxStep = ms;
    printf("Step: %lu  Updating max Step...dAcc: %lu,%lu   new maxStep: %.5G\n", mcs->sn,
           (unsigned long)st.d_acc[0], (unsigned long)st.d_acc[1], ms);
    report(jmm_plain_set_step_sizes(mcs->h, mcs->maxStep, mcs->maxdl), "jmm_plain_set_step_sizes");
  }
  return 0;
}

// maxDVAdjust (src/jmmMCState.cpp:2120-2139), including its clamp of values
// above 0.10 N to 0.50 N.
int maxDVAdjust(struct MCState *mcs) {
  static unsigned long int vAErrNtot = 0;
#pragma omp critical(jmm_dropin)
  {
    flush(mcs);
    const jmm_state st = state_of(mcs);
    const unsigned long int vtot = st.v_acc[0] + st.v_acc[1];
    if ((vtot - vAErrNtot) > 0) {
      vAErrNtot = vtot;
      const double ideal = 0.5;
      const double actual = (double)st.v_acc[0] / vtot;
      double md = mcs->maxdl * log(0.672924 * ideal + 0.0644284) /
                  log(0.672924 * (actual + 0.0644284));
      if (md < 0.002 * mcs->N)
        md = 0.002 * mcs->N;
      else if (md > 0.10 * mcs->N)
        md = 0.50 * mcs->N;
      mcs->maxdl = md;
      printf("Step: %lu  Updating max vol.ch....vAcc: %lu,%lu   new maxStep: %.5G\n", mcs->sn,
             (unsigned long)st.v_acc[0], (unsigned long)st.v_acc[1], md);
      report(jmm_plain_set_step_sizes(mcs->h, mcs->maxStep, mcs->maxdl),
             "jmm_plain_set_step_sizes");
    }
  }
  return 0;
}

// relaxVolume (src/jmmMCState.cpp:2396-2643): the Newton steps run on the
// GPU in one launch; their messages are printed from its per-step records.
int relaxVolume(struct MCState *mcs) {
  int rc = 0;
#pragma omp single copyprivate(rc)
  {
    flush(mcs);
    const jmm_state st = state_of(mcs);
    printf("Relaxing the Volume...Starting Length,Energy: %.5G,%.5G\n", st.l, st.tot[JMM_Q_E]);
    jmm_relax_step log[20];
    int32_t n = 0, conv = 0;
    report(jmm_plain_relax_volume(mcs->h, log, &n, &conv), "jmm_plain_relax_volume");
    for (int k = 0; k < n; ++k) {
      printf("Relaxation step %d...", k);
      if (k == n - 1 && conv)
        printf("Relaxation converged. Length,energy: %.10G,%.10G\n", log[k].l, log[k].e);
      else
        printf("length,energy: %.5g,%.5G\n", log[k].l, log[k].e);
    }
    if (!conv)
      printf("WARNING: Relaxation failed to converge after 20 steps. Length,energy: %.5G,%.5G\n",
             log[n - 1].l, log[n - 1].e);
    fflush(stdout);
    rc = conv ? 0 : 1;
  }
  return rc;
}

double calculateEnergyOfTrialVolumeChange(struct MCState *mcs, double dl) {
  double e = 0;
#pragma omp single copyprivate(e)
  {
    flush(mcs);
    report(jmm_plain_trial_volume_energy(mcs->h, dl, &e), "jmm_plain_trial_volume_energy");
  }
  return e;
}

int moveVolume(struct MCState *mcs, double l) {
#pragma omp single
  {
    flush(mcs);
    report(jmm_plain_move_volume(mcs->h, l), "jmm_plain_move_volume");
  }
  return (int)l;
}

unsigned long int getStepNum(struct MCState *mcs) { return mcs->sn; }
int getRelaxFlag(struct MCState *mcs) { return mcs->relaxFlag; }
bool getRestartFlag(struct MCState *mcs) { return mcs->isRestart; }

int printE(struct MCState *mcs) {
  flush(mcs);
  printf("\nE = %.8G\n", state_of(mcs).tot[JMM_Q_E]);
  return 0;
}

int printAcc(struct MCState *mcs) {
  flush(mcs);
  const jmm_state st = state_of(mcs);
  printf("Accepted/Rejected: Displacements VolumeChanges\n"
         "                        %lu/%lu          %lu/%lu\n",
         (unsigned long)st.d_acc[0], (unsigned long)st.d_acc[1], (unsigned long)st.v_acc[0],
         (unsigned long)st.v_acc[1]);
  return 0;
}
