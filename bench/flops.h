/* Algorithmic operation counts of the Tersoff + ILP force evaluation, frozen by
 * oracle/opcount.py: the oracle (oracle/lmff_oracle.c, pinned to the reference) compiled
 * with an operation-counting double (oracle/opcount.cpp), one evaluation of the
 * 36800-atom periodic patch of the 10-layer alternating-molecule graphite slab
 * (3.35 A, 300 K lattice, N(0, 0.03 A) displacement), BNC.tersoff + BNCH.ILP, 16 A, taper.
 * Convention: add, subtract, multiply, divide, sqrt = 1; a*b + c = 2; each exp, pow,
 * sin, cos call = 1 (CALLS_* counts them per unit, already inside FLOPS_*).
 * Generated file: regenerate with python oracle/opcount.py. */
#pragma once

/* an interlayer list candidate: displacement and r^2 (every candidate) */
#define LMFF_FLOPS_ILP_CAND 8.0000
#define LMFF_CALLS_ILP_CAND 0.0000
/* a directed pair in the cutoff, beyond the candidate's: r, taper, the repulsion term with the normal of i, forces on i and j, energy */
#define LMFF_FLOPS_ILP_PAIR 94.0000
#define LMFF_CALLS_ILP_PAIR 2.0000
/* one vdW evaluation (calc_FvdW, tag-parity half of the pairs) */
#define LMFF_FLOPS_ILP_VDW 41.0000
#define LMFF_CALLS_ILP_VDW 2.0000
/* calc_FRep's term of dn_i/dx_i (per pair; with the reverse-accumulated normal derivative it is applied once per atom) */
#define LMFF_FLOPS_ILP_DSELF 27.0000
#define LMFF_CALLS_ILP_DSELF 0.0000
/* calc_FRep's force on one intralayer neighbour k of i (per pair and k; applied once per atom and k with the reverse-accumulated normal derivative) */
#define LMFF_FLOPS_ILP_KTERM 27.0000
#define LMFF_CALLS_ILP_KTERM 0.0000
/* calc_normal of one atom: its normal and the Jacobians */
#define LMFF_FLOPS_NORMAL 270.0000
#define LMFF_CALLS_NORMAL 0.0000
/* Tersoff repulsive term of a bond (tag-parity half) */
#define LMFF_FLOPS_TERS_REP 25.0000
#define LMFF_CALLS_TERS_REP 1.0000
/* force_zeta and the bond force of a directed bond */
#define LMFF_FLOPS_TERS_BOND 61.0000
#define LMFF_CALLS_TERS_BOND 6.0000
/* zeta term of a triplet */
#define LMFF_FLOPS_TERS_ZETA 35.0000
#define LMFF_CALLS_TERS_ZETA 2.0000
/* three-body (attractive) force of a triplet */
#define LMFF_FLOPS_TERS_ATTR 196.5000
#define LMFF_CALLS_TERS_ATTR 3.0000
/* vdW evaluations per directed pair in the cutoff */
#define LMFF_VDW_PER_PAIR 0.5000
/* intralayer neighbours k of i per directed pair (k-terms of calc_FRep) */
#define LMFF_KTERMS_PER_PAIR 3.0000
/* Tersoff arithmetic per atom (repulsive + bond + zeta + attractive) */
#define LMFF_FLOPS_TERSOFF_ATOM 1609.5000
/* directed Tersoff bonds per atom */
#define LMFF_TERS_BONDS_PER_ATOM 3.0000
/* Tersoff triplets per atom */
#define LMFF_TERS_TRIPLETS_PER_ATOM 6.0000
/* directed interlayer pairs in the cutoff per atom */
#define LMFF_ILP_PAIRS_PER_ATOM 786.4951
/* interlayer list candidates per atom (the oracle's list: cutoff + 2 A skin) */
#define LMFF_ILP_CANDIDATES_PER_ATOM 1101.5617
