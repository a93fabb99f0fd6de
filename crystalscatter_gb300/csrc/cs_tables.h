// cs_tables.h — orientation quadrature node tables (internal).
//
// The orientation average of the reference is a nested Romberg integration:
// over the polar angle delta in [0, min(pi/2, dbeta*sqrt(ln 1e5))] and, for
// every delta node, over the azimuth chi in [0, 2*pi]
// (qrombdeltac/trapzddeltac and qrombchid/trapzdchid,
// Source/sc_calc_generic_gpu.cu:956-1583). The trapezoid nodes of refinement
// level j are x_1 = a + del/2, x_k = x_(k-1) + del with del = (b-a)/2^(j-2)
// (level 1 uses the end points). They do not depend on the pixel, so their
// sines, cosines and the Gaussian orientation weight sin(x)*exp(-x^2/dbeta^2)
// are evaluated once on the host, node by node in the reference's order, and
// the kernels read them from these tables. Levels beyond CS_NODE_LEVELS are
// evaluated on the fly.
#ifndef CS_TABLES_H
#define CS_TABLES_H

#define CS_NODE_LEVELS 16
/* nodes of levels 1..L: 2 + sum_{j=2..L} 2^(j-2) = 2^(L-1) + 1 */
#define CS_NODE_COUNT ((1 << (CS_NODE_LEVELS - 1)) + 1)

/* offset of the first node of refinement level j (j >= 1) */
#define CS_NODE_OFFSET(j) ((j) == 1 ? 0 : (1 << ((j)-2)) + 1)

typedef struct cs_chi_node {
    double c, s; /* cos(x), sin(x) */
} cs_chi_node;

/* FP32 copies of the chi nodes for the mixed-precision kernels: they follow the
 * CS_NODE_COUNT FP64 nodes in the same allocation (two per cs_chi_node slot),
 * so a chi table holds CS_CHI_TABLE_LEN cs_chi_node slots in all. */
typedef struct cs_chi_node_f {
    float c, s;
} cs_chi_node_f;
#define CS_CHI_TABLE_LEN (CS_NODE_COUNT + (CS_NODE_COUNT + 1) / 2)

typedef struct cs_delta_node {
    double w;    /* sin(x)*exp(-x*x/(dbeta*dbeta)) */
    double c, s; /* cos(x), sin(x) */
} cs_delta_node;

#endif
