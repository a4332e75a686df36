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
 *   gctr                 Cartesian accumulators, CGTask::cart_off, layout [comp][nf]
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
    int sym;             /* unique-quartet flags: bit0 I != J, bit1 K != L, bit2 IJ != KL */
    int cls;             /* adjoint only: index of the class's iteration tables (CGGradClass) */
    int pad;
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

typedef struct {
    int64_t cart_off;    /* first accumulator slot; nparts slots follow, each ncomp*nf long */
    int64_t out_off;     /* element offset in the output array */
    int st[4];           /* output strides of the four shell indices (kernel order I,J,K,L) */
    int l[4];            /* angular momenta in kernel order */
    int nparts;
    int flags;           /* bit0: 1 = spherical output */
} CGOutTask;

#endif
