/*
 * cs_prepared.h — layout of one prepared parameter set ("constant block").
 *
 * The host preparation (cs_prep.cpp) turns a cs_params into this block: the
 * flags, image geometry, Schulz-Zimm series coefficients, series/asymptote
 * switch points (limq*), orientation norm and the lattice reflection tables of
 * the reference's prepareCalculation()/coefficients()
 * (Source/sc_calc_generic_cpu.cpp:319-988, 2099-8195). The block is plain C so
 * that the CUDA kernels, the C ABI and the CPU test oracle read one layout.
 * Array dimensions follow the reference: coefficient arrays [0..150]
 * (coeffarray_len, sc_calc_generic_gpu.h:443), carr11pm [131][131]
 * (imax2d_len, :444), reflection tables latpar1/2 int[2500][6] and latpar3
 * float[2500][17] (:543-561).
 */
#ifndef CS_PREPARED_H
#define CS_PREPARED_H

#define CS_COEFF_LEN 151
#define CS_IMAX2D 131
#define CS_LATPARLEN 2500

/* Quadrant codes as in the reference _radQX (Source/sc_math.h:26-31). */
#define CS_RADQ1 0
#define CS_RADQ2 1
#define CS_RADQ4 2
#define CS_RAD1D 3

/* Orientation case, 0-based exactly like the reference's _orcaseType
   (sc_calc_generic_gpu.h:487-493); the library functions compare it with the
   1-based integers of the original Pascal code, which is reproduced. */
#define CS_ORC_GENERAL 0
#define CS_ORC_XAXIS 1
#define CS_ORC_YAXIS 2
#define CS_ORC_ZAXIS 3

/* Dispatch keys (particle<<24 | shp<<16 | ltype<<8 | ordis), the reference's
   specialised pixel functions (Source/sc_calc_generic_gpu.cu:113-132). */
#define CS_KEY_SPHERE_NONE_ISO 0x00000C07
#define CS_KEY_SPHERE_GAUSS_FCC_GAUSS 0x00020500
#define CS_KEY_CYL_NONE_GAUSS 0x01000C00
#define CS_KEY_CYL_NONE_ZDIR 0x01000C06
#define CS_KEY_CYL_GAUSS_BCT_ZDIR 0x01020806
#define CS_KEY_CUBE_NONE_ISO 0x04000C07
/* every other combination, and every combination with bIgnoreNewSwitch: the
   reference's calc_GENERIC (Source/sc_gpu_generic.h:27-881) */
#define CS_KEY_GENERIC 0x7F000000

typedef struct cs_prepared {
    /* dispatch */
    int key;         /* switch key of kernel_selection / calcCPU_selection */
    int ign_switch;  /* bIgnoreNewSwitch */
    int particle, shp, ltype, ordis, cs, part, cdim, partdim, orcase;
    int lattice, twin, debyescherrer, para;

    /* image geometry (convert_idx2q, Source/sc_calc_generic_gpu.cu:249-287) */
    int use1d, usebeamstop, zmax;
    int zzmin, zzmax, iimin, iimax; /* calculated index range */
    int xmin, xmax, ymin, ymax;     /* image extents (checkArrays) */
    int calc_quadrants, expand;
    double qmax, qmin, pixnox, pixnoy, pixx_m, pixy_m, beamx0, beamy0, det, wave;

    /* pixel manipulation */
    double base, izero, iso, ifluc, rfluc;

    /* particle (params.* after preparation) */
    double radius, radiusi, sigma, sigmal, length, p1, rho, alphash1, alpha, poltheta, polphi, dbeta;
    double norm, por, order;
    double limq[10];  /* limq1..limq9 at [1..9] */
    double limqf[10]; /* limq1f..limq9f at [1..9] */
    double cosphic, sinphic, cosphi, sinphi, costheta, sintheta;
    double sig[3];
    double ax1[3], ax2[3], ax3[3];
    /* gamma(zr-1/2)/gamma(zr+1) and gamma(zr-3/2)/gamma(zr+1) with the
       reference's gamma(): pixel-independent factors of the cylinder F(q)
       asymptote, evaluated once on the host */
    double gamma_ratio[2];
    /* orientation quadrature of formpq/formfq_partCylinder for ordis 0
       (qrombdeltac(..., theta=polTheta, phi=0, i0=4, i1=orcase)): the upper
       limits as the reference stores them (float blim, widened to double),
       dbeta in radians and the float-rounded direction matrix p11..p33 */
    double romb_delta_b, romb_chi_b, romb_dbeta;
    double romb_p[9];

    /* lattice */
    int peakmax1, peakmax2;
    double latpar[4]; /* [1]=ucvol [2]=sphno [3]=dwfactor */
    double dwfactor, uca, ucb, domainsize, width_zuf, reldis, dist, phiwidth, ceff;

    /* coefficient arrays: carrp[k] = carr(k+1)p, carrf[k] = carr(k+1)f */
    double carrp[9][CS_COEFF_LEN];
    double carrf[9][CS_COEFF_LEN];
    double carr11pm[CS_IMAX2D][CS_IMAX2D];

    /* reflection tables */
    int latpar1[CS_LATPARLEN][6];
    int latpar2[CS_LATPARLEN][6];
    float latpar3[CS_LATPARLEN][17];

    /* 2D-fit masks (checkFitRanges, Source/sc_calc_generic_gpu.cu:293-347) */
    int nofit_x0[4], nofit_x1[4], nofit_y0[4], nofit_y1[4];
    int fit_width, fit_height, fit_bstop, fit_border;

    /* peak-shape constants of the generic lattice sums (prepareCalculation,
       Source/sc_calc_generic_cpu.cpp:585-590, and setPeakPar: eta = peakpar/100,
       beta = peakpar); gamma(beta) and gamma(beta - 1/2) for Pearson VII */
    double pk_c1, pk_c2, pk_c3, pk_c4, pk_eta, pk_beta, pk_gbeta, pk_gbeta_h;
} cs_prepared;

#endif /* CS_PREPARED_H */
