"""Formatting of the reference's thermo block averages.

printThermo (src/jmmMCState.cpp:1896-1937) divides the 12 accumulators by
the steps since the last print and writes
``sn\\tEconf\\tEconf2\\tL\\tL2\\tLEconf\\trho\\trho2\\tVirial\\tVirial2\\tEconfVir\\tHV\\tHV2``
with ``%.8G``; the accumulator order of include/jmm_gpu.h is rhoSysA,
rhoSysSA, lA, lSA, EA, ESA, lEA, VirA, VirSA, EVirA, HVA, HVSA.
"""

HEADER = ("Step    Econf           Econf2          L       L2      LEconf          "
          "rho             rho2            Virial         Virial2         "
          "EconfVir        HV              HV2 \n")

# file column -> accumulator index
_COLUMN_ORDER = (4, 5, 2, 3, 6, 0, 1, 7, 8, 9, 10, 11)


def thermo_line(sn, acc, ss):
    means = [acc[k] / ss for k in _COLUMN_ORDER]
    return f"{sn}" + "".join("\t%.8G" % m for m in means) + "\n"


def rho_line(sn, counts, ns, rbw):
    """One line of rho.dat.mcs (printRho, src/jmmMCState.cpp:1021-1037): the
    step, then per bin the accumulated count / ns / rbw with %.8G; ns is the
    steps since the last print as an unsigned 64-bit difference."""
    ns = float(ns)
    return f"{sn}" + "".join(" %.8G" % (float(c) / ns / rbw) for c in counts) + "\n"


def g_line(sn, counts, ns, gsw, gbw):
    """One line of g<k>.dat.mcs (printG, src/jmmMCState.cpp:1042-1061): per
    separation bin of slice k, count / ns / gsw / gbw with %.8G."""
    ns = float(ns)
    return f"{sn}" + "".join(" %.8G" % (float(c) / ns / gsw / gbw) for c in counts) + "\n"
