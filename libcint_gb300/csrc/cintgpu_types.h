/*
 * Data layout shared by the host planner (cintgpu_host.cpp) and the CUDA kernels
 * (rys_kernels.cu).  Everything the kernels read lives in HBM in these flat arrays:
 *
 *   CGPair[npair]        one ordered shell pair (A, B); A is the recurrence base centre
 *   CGPrimPair[nprim]    its primitive pairs, ip fastest (jp * npa + ip), libcint's loop order
 *                        (src/cint2e.c:400-425); contraction coefficients are folded into K
 *   CGTask[ntask]        one unit of kernel work: bra pair, ket pair and a slice of the surviving
 *                        primitive quartets (pqlist)
 *   CGOutTask[nout]      one contracted shell quartet to transform (cart -> sph) and store
 *   CGEriClass/CGEriGroup/... per-class tables of the contraction-first kernel and the transfer
 *   CGGradClass/...      per-class tables of the adjoint
 *   gctr                 accumulator slots, CGTask::cart_off: (e0|f0) in group layout (int2e,
 *                        int3c2e) or Cartesian [comp][nf] (per-primitive classes, int2e_ip1)
 */
#ifndef CINTGPU_TYPES_H
#define CINTGPU_TYPES_H
#include <stdint.h>

#define CG_MAXL      8     /* largest angular momentum of a g-array axis (l + derivative) */
#define CG_MAX_SHELL_L 6   /* largest shell angular momentum accepted by the drop-in */

typedef struct {
    double AB[3];        /* R_A - R_B (horizontal transfer vector) */
    double A[3];         /* R_A (vertical recurrence base) */
    int prim_off;        /* first CGPrimPair */
    int npa, npb;        /* primitive counts of A and B */
    int la, lb;          /* angular momenta */
    int ao_a, ao_b;      /* Cartesian AO offsets of A and B (J contraction, adjoint) */
    int atom_a, atom_b;  /* atoms of A and B (adjoint) */
    int gp_a, gp_b;      /* first global primitive index of A and B (exponent adjoint) */
    int pad;
} CGPair;

typedef struct {
    double a;            /* a_A + a_B */
    double inv_a;        /* 1 / (a_A + a_B) */
    double P[3];         /* Gaussian product centre */
    double K;            /* c_A c_B exp(-a_A a_B / (a_A + a_B) |AB|^2) */
    double cce;          /* libcint screening value (src/optimizer.c:301-338) */
    double aA;           /* exponent on centre A (needed by the nabla of int2e_ip1) */
} CGPrimPair;

typedef struct {
    int pij, pkl;        /* bra / ket pair indices */
    int pq_off, npq;     /* surviving primitive quartets pqlist[pq_off .. pq_off+npq),
                            each encoded kl * nij + ij */
    int64_t cart_off;    /* accumulator slot in gctr */
    int out;             /* CGOutTask index (for the non-empty flag) */
    int sym;             /* unique-quartet flags: bit0 I != J, bit1 K != L, bit2 IJ != KL;
                            per-primitive kernels: bit3 (bit4) runs the bra (ket) recurrences
                            about the pair's second centre (see g_axis) */
    int cls;             /* class tables: CGGradClass (adjoint) or CGEriClass (int2e, int3c2e, J) */
    int own_slot;        /* 1: the quartet's only slice accumulates in the running warp's slot
                            (CGLaunch::wslot), not at cart_off, and that warp transforms it */
} CGTask;

/* Adjoint iteration tables, one set per angular-momentum class, built on the host.
 * For axis a and a-axis power tuple u, the components sharing u are the entries
 * ent[chunk.ent .. chunk.ent + chunk.len): offsets of the partner axes' g values and the
 * component index into the cotangent W.  Chunks hold <= 16 entries, sorted longest first. */
typedef struct { int chunk_off, nchunk, pad0, pad1; } CGGradClass;
typedef struct {
    int axis_u;          /* axis | u << 2 */
    int ent, len;        /* entries [ent, ent + len) */
    int ou;              /* offset of tuple u in the axis's g array */
    int om[3];           /* offset of u lowered on shell I, J, K (= ou where that power is 0) */
    int pad;
    double p[3];         /* powers of u on shells I, J, K (as doubles: no conversion in the kernel) */
} CGGradChunk;
typedef struct { int ob_oc; int c; } CGGradEnt;                          /* ob | oc << 16 */

/* Contraction-first int2e/int3c2e tables, one set per angular-momentum class (kernel order,
 * li >= lj, lk >= ll).  The kernel accumulates (e0|f0) = sum over primitive quartets and roots of
 * gx gy gz for every Cartesian e = (ex,ey,ez) with li <= |e| <= li+lj and f likewise, and the
 * horizontal transfer to (ij|kl) runs once per contracted quartet.  A group is one
 * (ex, ey, fx, fy): the product gx gy is formed once and multiplies gz for each (ez, fz) member.
 * Accumulator layout: row baseE(ex,ey) + (ez - ez0), column baseF(fx,fy) + (fz - fz0), nF columns;
 * eperm/fperm map the transfer's Cartesian order (shells ascending, libcint order within a shell)
 * to those rows/columns.  Classes with bra = 1 replace e by the Cartesian pair (i, j) of the bra
 * shells: a group is one (ix jx, iy jy, fx, fy), its z powers of i and j are fixed, so it has one
 * row (i nfj + j) and the nfz members of f. */
typedef struct {
    int group_off, ngroup;   /* CGEriGroup range, ordered by shape (nez, nfz) */
    int perm_off;            /* eperm[nE] then fperm[nF] */
    int nE, nF;
    int split;               /* ngroup <= 32: lanes per group (power of two); 0: groups in rounds */
    int hrr_need;            /* doubles of each of the two transfer buffers */
    int maxab;               /* (lj + 1) | (ll + 1) << 8: member box of the class */
    int hprog_off;           /* horizontal-transfer program (ints), see cg_hrr */
    int round_off, nround;   /* stage-3 rounds (ints: first group | count << 16 | box << 24,
                                box = (MA-1) + 4 (MB-1) of the round's largest nez, nfz) */
    int bra;                 /* 1: the bra transfer runs per term on each axis's 2D integrals
                                (libcint's order on the bra), the accumulators hold (ij|f0) with
                                rows i nfj + j, and only the ket transfer follows contraction */
} CGEriClass;
typedef struct {
    int oxy;             /* ox | oy << 16: offsets of (ex, fx) and (ey, fy) in the VRR arrays */
    int oz;              /* offset of (ez0, fz0) in the z array */
    int acc;             /* accumulator index of member (0, 0) */
    int mn;              /* nez | nfz << 8 */
} CGEriGroup;

typedef struct {
    int64_t cart_off;    /* first accumulator slot; nparts slots follow, each ncomp*nf long
                            (nE*nF with flags bit1) */
    int64_t out_off;     /* element offset in the output array */
    int st[4];           /* output strides of the four shell indices (kernel order I,J,K,L) */
    int l[4];            /* angular momenta in kernel order */
    int nparts;
    int flags;           /* bit0: 1 = spherical output; bit1: slots hold (e0|f0) of class ecls */
    int ecls;
    int pad;
    double AB[3], CD[3]; /* transfer vectors R_I - R_J, R_K - R_L */
} CGOutTask;

#endif
