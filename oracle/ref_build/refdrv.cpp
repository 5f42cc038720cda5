/*
 * refdrv.cpp -- driver for the reference build (test infrastructure).
 *
 * Runs the reference's own one-component loop (fJmodels.cpp:86-144) with the
 * radial grid taken from the command line instead of SetGrid(200.), and dumps
 * every intermediate at full precision so the oracle can be checked against
 * the reference code itself.
 *
 *   refdrv <param file> <rmin> <rmax> <points file or -> <dump file>
 *
 * Points file lines: "P R z" (potential and gradient), "A R z vR vphi vz"
 * (actions with Delta from the table, as df() does), "M R z" (rhofDF),
 * "S R z" (SigmaDF), "L R z vx" (line_profile), "F R z vphi" (P_vp),
 * "Z R z vz" (P_vz), "X R z vR" (P_vr), all in the guess potential with the
 * guess density multipoles.
 * FJREF_DELTA_FILE, when set, names a file with a focal-distance table
 * (Egrid then Dgrid) used instead of tabulateDelta.
 *
 * A parameter file with a second component runs the reference's two-component
 * loop instead (twoComp, fJmodels.cpp:38-81, in its own order: component 1's
 * moments in the total potential, whose own new potential then replaces the
 * total, component 2's in that, total = the sum) and dumps each component's
 * matrices and the total potential per iteration; the points file is unused.
 */
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>
#include "Utils.h"
#include "UtilsLeg.h"
#include "readParam.h"
#include "Potential.h"
#include "models.h"
#include "Delta.h"
#include "Tabulate.h"
#include "uvOrb.h"
#include "DF.h"
#include "Integ.h"
#include "potLeg.h"
#include "Stats.h"
#include "writeOut.h"

double ar[NR], Dgrid[NGRID], Egrid[NGRID];
double ** __restrict phil, ** __restrict Pr, ** __restrict Pr2,
       ** __restrict rhl, ** __restrict vrotl, ** __restrict sigRl,
       ** __restrict sigpl, ** __restrict sigzl, ** __restrict sigRzl;
FILE * __restrict f_lz;

static FILE *out;
extern unsigned components;  // io/readParam.cpp:16
static void dumpv(const char *name, const double *v, int n)
{
    fprintf(out, "%s %d\n", name, n);
    for (int i = 0; i < n; i++) fprintf(out, "%.17g\n", v[i]);
}
static void dumpm(const char *name, double **m, int nx, int ny)
{
    fprintf(out, "%s %d\n", name, nx * ny);
    for (int i = 0; i < nx; i++)
        for (int j = 0; j < ny; j++) fprintf(out, "%.17g\n", m[i][j]);
}

static int two_components(struct fJParams fJP)
{
    double **rhl2 = mat<double>(NR, NPOLY), **vrotl2 = mat<double>(NR, NPOLY), **sigRl2 = mat<double>(NR, NPOLY),
           **sigpl2 = mat<double>(NR, NPOLY), **sigzl2 = mat<double>(NR, NPOLY), **sigRzl2 = mat<double>(NR, NPOLY);
    SetModel(fJP, 1);
    Potential p(1);
    p.selectGuessRho(fJP.modName != "null" ? fJP.modName : "Hernquist");
    p.computeGuessRhl();
    p.computePhil(p.rhlP);
    SetModel(fJP, 2);
    Potential p2(2);
    p2.selectGuessRho(fJP.modName2 != "null" ? fJP.modName2 : "Hernquist");
    p2.computeGuessRhl();
    p2.computePhil(p2.rhlP);
    updatePhil(&p, &p2);
    dumpm("c1_guess_rhl", p.rhlP, NR, NPOLY);
    dumpm("c2_guess_rhl", p2.rhlP, NR, NPOLY);
    dumpm("guess_phil", phil, NR, NPOLY);
    dumpm("guess_Pr", Pr, NR, NPOLY);
    dumpm("guess_Pr2", Pr2, NR, NPOLY);
    const char *dfile = getenv("FJREF_DELTA_FILE");
    if (dfile) {
        FILE *df = fopen(dfile, "r");
        for (int i = 0; i < NGRID; i++) if (fscanf(df, "%lf", &Egrid[i]) != 1) return 3;
        for (int i = 0; i < NGRID; i++) if (fscanf(df, "%lf", &Dgrid[i]) != 1) return 3;
        fclose(df);
    } else tabulateDelta(&p);
    dumpv("Egrid", Egrid, NGRID);
    dumpv("Dgrid", Dgrid, NGRID);
    fflush(out);
    char nm[64];
    for (int k = 0; k < fJP.itermax; k++) {
        printf("\n Iter:%d\n", k);
        setDF(&fJP, &p, 1);
        computeNewPhi(&p, rhl, sigRl, sigpl, sigzl, sigRzl, vrotl);
        setDF(&fJP, &p, 2);
        computeNewPhi(&p2, rhl2, sigRl2, sigpl2, sigzl2, sigRzl2, vrotl2);
        updatePhil(&p, &p2);
        double **m1[9] = {rhl, vrotl, sigRl, sigpl, sigzl, sigRzl, p.philP, p.PrP, p.Pr2P};
        double **m2[9] = {rhl2, vrotl2, sigRl2, sigpl2, sigzl2, sigRzl2, p2.philP, p2.PrP, p2.Pr2P};
        const char *names[9] = {"rhl", "vrotl", "sigRl", "sigpl", "sigzl", "sigRzl", "phil", "Pr", "Pr2"};
        for (int q = 0; q < 9; q++) {
            snprintf(nm, sizeof nm, "it%d_c1_%s", k, names[q]); dumpm(nm, m1[q], NR, NPOLY);
            snprintf(nm, sizeof nm, "it%d_c2_%s", k, names[q]); dumpm(nm, m2[q], NR, NPOLY);
        }
        double **tot[3] = {phil, Pr, Pr2};
        for (int q = 0; q < 3; q++) { snprintf(nm, sizeof nm, "it%d_%s", k, names[6 + q]); dumpm(nm, tot[q], NR, NPOLY); }
        fflush(out);
    }
    fclose(out);
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 6) { fprintf(stderr, "usage: refdrv param rmin rmax points dump\n"); return 2; }
    phil = mat<double>(NR, NPOLY); Pr = mat<double>(NR, NPOLY); Pr2 = mat<double>(NR, NPOLY);
    rhl = mat<double>(NR, NPOLY); vrotl = mat<double>(NR, NPOLY);
    sigRl = mat<double>(NR, NPOLY); sigpl = mat<double>(NR, NPOLY);
    sigzl = mat<double>(NR, NPOLY); sigRzl = mat<double>(NR, NPOLY);
    struct fJParams fJP = readParam(argv[1]);
    double rmin = atof(argv[2]), rmax = atof(argv[3]);
    for (int i = 0; i < NR; i++) ar[i] = pow(10., log10(rmin) + (log10(rmax) - log10(rmin)) * i / (NR - 1));
    out = fopen(argv[5], "w");
    f_lz = fopen("/dev/null", "w");
    std::vector<std::vector<double>> pts;
    if (strcmp(argv[4], "-")) {
        std::ifstream pf(argv[4]);
        std::string line;
        while (std::getline(pf, line)) {
            std::stringstream ss(line);
            char t;
            ss >> t;
            std::vector<double> v{(double)t};
            double x;
            while (ss >> x) v.push_back(x);
            if (v.size() > 1) pts.push_back(v);
        }
    }
    dumpv("ar", ar, NR);
    if (components == 2) return two_components(fJP);

    SetModel(fJP);
    Potential p;
    p.selectGuessRho(fJP.modName != "null" ? fJP.modName : "Hernquist");
    p.computeGuessRhl();
    p.computePhil();
    dumpm("guess_rhl", rhl, NR, NPOLY);
    dumpm("guess_phil", phil, NR, NPOLY);
    dumpm("guess_Pr", Pr, NR, NPOLY);
    dumpm("guess_Pr2", Pr2, NR, NPOLY);

    std::vector<double> pv;
    for (auto &v : pts)
        if ((char)v[0] == 'P') { pv.push_back(p(v[1], v[2])); pv.push_back(p.dR(v[1], v[2])); pv.push_back(p.dz(v[1], v[2])); }
    dumpv("pot_points", pv.data(), (int)pv.size());

    const char *dfile = getenv("FJREF_DELTA_FILE");
    if (dfile) {  /* use a given focal-distance table (2*NGRID values: Egrid then Dgrid) */
        FILE *df = fopen(dfile, "r");
        for (int i = 0; i < NGRID; i++) if (fscanf(df, "%lf", &Egrid[i]) != 1) return 3;
        for (int i = 0; i < NGRID; i++) if (fscanf(df, "%lf", &Dgrid[i]) != 1) return 3;
        fclose(df);
    } else tabulateDelta(&p);
    dumpv("Egrid", Egrid, NGRID);
    dumpv("Dgrid", Dgrid, NGRID);

    setDF(&fJP, &p, 1);
    std::vector<double> av, mv, lv;
    for (auto &v : pts) {
        switch ((char)v[0]) {
        case 'S': lv.push_back(SigmaDF(v[1], v[2])); break;
        case 'L': lv.push_back(line_profile(v[1], v[2], v[3], &p)); break;
        case 'F': lv.push_back(P_vp(v[1], v[2], v[3], &p)); break;
        case 'Z': lv.push_back(P_vz(v[1], v[2], v[3], &p)); break;
        case 'X': lv.push_back(P_vr(v[1], v[2], v[3], &p)); break;
        default: break;
        }
        if ((char)v[0] == 'A') {
            double x[3] = {v[1], v[2], p(v[1], v[2])}, vel[2] = {v[3], v[5]};
            double H = .5 * (v[3] * v[3] + v[4] * v[4] + v[5] * v[5]) + x[2];
            if (H >= 0) { av.push_back(-1); av.push_back(-1); continue; }
            uvOrb o(Deltafn(H), v[1] * v[4], x[2], x, vel, &p);
            av.push_back(o.Ju());
            av.push_back(o.Jv());
        } else if ((char)v[0] == 'M') {
            double vr, sR, sp, sz, sRz;
            double d = rhofDF(v[1], v[2], &p, &vr, &sR, &sp, &sz, &sRz);
            double m6[6] = {d, vr, sR, sp, sz, sRz};
            for (double q : m6) mv.push_back(q);
        }
    }
    dumpv("actions", av.data(), (int)av.size());
    dumpv("moments", mv.data(), (int)mv.size());
    dumpv("los", lv.data(), (int)lv.size());
    fflush(out);

    for (int k = 0; k < fJP.itermax; k++) {
        printf("\n Iter:%d\n", k);
        computeNewPhi(&p, rhl, sigRl, sigpl, sigzl, sigRzl, vrotl);
        char nm[64];
        double **mats[9] = {rhl, vrotl, sigRl, sigpl, sigzl, sigRzl, phil, Pr, Pr2};
        const char *names[9] = {"rhl", "vrotl", "sigRl", "sigpl", "sigzl", "sigRzl", "phil", "Pr", "Pr2"};
        for (int q = 0; q < 9; q++) { snprintf(nm, sizeof nm, "it%d_%s", k, names[q]); dumpm(nm, mats[q], NR, NPOLY); }
        fflush(out);
        writeOut(fJP, k, &p);
        vir2(&p);
        fflush(stdout);
    }
    fclose(out);
    return 0;
}
