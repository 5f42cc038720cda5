/* Forced include for building the reference at run-time-chosen grid sizes
   (test infrastructure).  It provides what include/Grid.h provides, with
   NR/NGAUSS/NPOLY taken from -DREF_NR/-DREF_NGAUSS/-DREF_NPOLY, and defines
   Grid.h's include guard so the original body is skipped. */
#ifndef INCLUDE_GRID_H_
#define INCLUDE_GRID_H_
#define NR REF_NR
#define NGRID 30
#define NGAUSS REF_NGAUSS
#define NPOLY REF_NPOLY
extern double ar[NR], Dgrid[NGRID], Egrid[NGRID];
extern double ** __restrict phil, ** __restrict Pr, ** __restrict Pr2,
              ** __restrict rhl, ** __restrict vrotl, ** __restrict sigRl,
              ** __restrict sigpl, ** __restrict sigzl, ** __restrict sigRzl;
extern unsigned components;
#endif
