/*
 * Algorithmic work per unit of the induced-dipole path, used for every
 * roofline figure (bench.py reads the same numbers).  Counts are per ordered
 * pair / per operator application and exclude the arithmetic the reference
 * does not do (self pairs, excluded pairs, padding).
 *
 *   damped dipole pair     45 FLOP + 2 MUFU (rsqrt, exp):
 *                          r (3) + r^2 (5) + R (1) + v = a s_i s_j R (2) +
 *                          f_E, f_T (8) + R^-3, R^-5 (3) + mu.r (5) + scale (3) +
 *                          field update (13), with 1 FLOP for the exp argument
 *   undamped dipole pair   31 FLOP + 1 MUFU
 *   charge pair            14 FLOP + 1 MUFU
 *   quadrupole pair        ~70 FLOP + 1 MUFU
 *   M2L (dipole sources)   order 5: 863 FLOP, order 6: 1731 FLOP
 *   CG iteration (HBM)     ~12 passes over 3N values (x, r, z, p, Ap) + apply traffic
 */
#ifndef CPPE_GPU_WORK_MODEL_H
#define CPPE_GPU_WORK_MODEL_H

#define CPPE_WORK_DAMPED_DIPOLE_PAIR_FLOP 45
#define CPPE_WORK_DIPOLE_PAIR_FLOP 31
#define CPPE_WORK_CHARGE_PAIR_FLOP 14
#define CPPE_WORK_QUADRUPOLE_PAIR_FLOP 70
#define CPPE_WORK_M2L_DIPOLE_P5_FLOP 863
#define CPPE_WORK_M2L_DIPOLE_P6_FLOP 1731

#endif
