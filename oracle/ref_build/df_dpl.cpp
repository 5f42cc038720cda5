/*
 * df_dpl.cpp -- test infrastructure for the reference build.
 *
 * The reference's df() (df/DF.cpp:78-124) returns the quasi-isothermal DF
 * at DF.cpp:106; its double-power-law DF with the tanh(chi*Jphi/J0) rotation
 * term (DF.cpp:108-119) is unreachable.  This file stands in for DF.cpp when
 * the reference is built for the double-power-law DF: the slope selection of
 * setDF (DF.cpp:36-63), df_hg (DF.cpp:72-76) and the rotation term are
 * re-expressed so that branch runs, with k taken from FJREF_K (DF.cpp:109
 * hard-codes k=1).  Everything else (actions, Delta lookup) is the
 * reference's own code.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <math.h>
#include "DF.h"
#include "models.h"
#include "readParam.h"
#include "Tabulate.h"
#include "Utils.h"
#include "uvOrb.h"

static double slope[2] = {5. / 3., 5.};
static double dph_h, dzz_h, dph_g, dzz_g, kRot = 1.0;
static Potential *gPot;

void setDF(const double a, const double b, const double c, const double d, Potential *p)
{
    gPot = p;
    dph_h = a; dzz_h = b; dph_g = c; dzz_g = d;
}

void setDF(struct fJParams *fJP, Potential *p, const unsigned comp)
{
    const char *ks = getenv("FJREF_K");
    kRot = ks ? atof(ks) : 1.0;
    std::string name = comp == 1 ? fJP->modName : fJP->modName2;
    double A = comp == 1 ? fJP->alpha : fJP->alpha_2, B = comp == 1 ? fJP->beta : fJP->beta_2;
    if (name == "Hernquist") { A = 1.667; B = 5.; }
    else if (name == "Isochrone") { A = 0.0; B = 5.; }
    else if (name == "NFW") { A = 1.667; B = 3.; }
    if (comp == 1) { fJP->alpha = A; fJP->beta = B; } else { fJP->alpha_2 = A; fJP->beta_2 = B; }
    slope[0] = A; slope[1] = B;
    if (comp == 1) {
        J0 = sqrt(fJP->mass * fJP->r0); mass = fJP->mass; chi = fJP->chi;
        setDF(fJP->dphi_h_in, fJP->dz_h_in, fJP->dphi_g_in, fJP->dz_g_in, p);
    } else {
        J0 = sqrt(fJP->mass_2 * fJP->r0_2); mass = fJP->mass_2; chi = fJP->chi_2;
        setDF(fJP->dphi_h_in2, fJP->dz_h_in2, fJP->dphi_g_in2, fJP->dz_g_in2, p);
    }
}

double df(const double *x, const double *v)
{
    double R = x[0], Lz = R * v[1], Phi_h = x[2];
    double H = .5 * (pow(v[0], 2) + pow(v[1], 2) + pow(v[2], 2)) + Phi_h;
    if (H >= 0) return 0.;
    double p[2] = {v[0], v[2]}, Jr, Jphi, Jz;
    uvOrb uvorb(Deltafn(H), Lz, Phi_h, x, p, gPot);
    Jr = uvorb.Ju(); Jz = uvorb.Jv(); Jphi = Lz;
    double h = Jr + dph_h * fabs(Jphi) + dzz_h * Jz, g = Jr + dph_g * fabs(Jphi) + dzz_g * Jz;
    double DFeven = mass / pow(J0, 3) * MAX(0., pow(1. + J0 / h, slope[0]) / (pow(1. + g / J0, slope[1]))) / (pow(TPI, 3.));
    double DF = chi == 0. ? DFeven : DFeven + kRot * tanh(chi * Jphi / J0) * DFeven;
    if (isnan(DF)) return 0.;
    return DF;
}
