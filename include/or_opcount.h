/* or_opcount.h -- algorithmic FP32 operations per unit of work of the YZ
 * tracklet stage, hand-counted from the reference's source and frozen here.
 *
 * Counting rule: every FP32 add, subtract, multiply, divide, square root,
 * absolute value, min/max and comparison is one operation; negation,
 * integer arithmetic and int-to-float conversions are not counted; a
 * short-circuit condition counts all of its comparisons.  The counts are
 * those of the reference's algorithm (which, for instance, recomputes every
 * hit's y for every combination), not of this library's kernels, which
 * hoist such work out of the combination loop: they define the work a
 * combination represents, as algorithmic bytes do for a memory-bound kernel.
 *
 * Units (reconstruction_kernels.cuh, "K"; reconstruction_helper.cuh, "H";
 * trackanalyticalminimizer.cuh, "AM"; trackfittingtools.cuh, "FT"):
 *
 *   fitted combination (u3, v3, u2, v2) with n accepted u/v hits: a y per
 *   hit (calculate_y_uvhit, H:75-100), the weighted line fit
 *   (fit_2D_track, AM:32-74, with matinv_2x2_matrix_per_thread, FT:3-82)
 *   and the 2-sigma cut (K:1611):
 *       OR_OPS_YZ_FIRST(n) = n*(OR_OPS_CALC_Y + OR_OPS_FIT_POINT) + OR_OPS_FIT_FIXED + OR_OPS_YZ_CUT1
 *
 *   survivor of that cut with n u/v hits and nx x hits: left/right
 *   resolution of the adjacent pairs (resolve_leftright_newhits, K:1615,
 *   H:714-780; about n/2 pairs) and of the single hits
 *   (resolve_single_leftright_newhits, H:785-804), the refit (K:1628), the
 *   hard cut (K:1638), the prop-tube y match (K:1640-1702, one check per
 *   prop plane), the three hodoscope matches (match_tracklet_to_hodo,
 *   H:1002-1087, the expected position and window per station) and
 *   chi2_track over the x and u/v hits (H:1182-1204 with residual,
 *   H:1149-1165):
 *       OR_OPS_YZ_SURVIVOR(n, nx) = (n/2)*OR_OPS_LR_PAIR + n*OR_OPS_LR_SINGLE
 *           + n*OR_OPS_FIT_POINT + OR_OPS_FIT_FIXED + OR_OPS_YZ_CUT2
 *           + OR_OPS_PROP_MATCH + OR_OPS_HODO_MATCH + (n + nx)*OR_OPS_CHI2_HIT
 */
#ifndef OR_OPCOUNT_H
#define OR_OPCOUNT_H

/* calculate_y_uvhit, hit sign 0 (H:75-100): wire end points 2+2, p2x 1,
 * x_trk 2, the two overlap tests 3+3, y 4, clamp 3, err_y 3 */
#define OR_OPS_CALC_Y 23
/* fit_2D_track per point (AM:46-56 normal sums 13, AM:69-72 chi2 sum 8) */
#define OR_OPS_FIT_POINT 21
/* fit_2D_track per fit: the 2x2 inverse with pivot search 13 (FT:25-80),
 * parameters 8 and errors 4 (AM:59-66) */
#define OR_OPS_FIT_FIXED 25
/* |y0| > Y0_MAX + 2 err_y0 || |ty| > TY_MAX + 2 err_ty (K:1611) */
#define OR_OPS_YZ_CUT1 8
/* one adjacent pair of resolve_leftright_newhits: expected slope and
 * intercept with their errors 16, four hypotheses of 24 (positions 4, local
 * slope 3, intercept 2, window 4, pull 10, minimum 1), the final test 1 */
#define OR_OPS_LR_PAIR 113
/* one hit of resolve_single_leftright_newhits: expected position 7, test 1 */
#define OR_OPS_LR_SINGLE 8
/* |y0| > Y0_MAX || |ty| > TY_MAX (K:1638) */
#define OR_OPS_YZ_CUT2 4
/* prop-tube y match: y expected and distance test, 5 per plane, 4 planes */
#define OR_OPS_PROP_MATCH 20
/* hodoscope matches: expected position and window, 10 per station, 3 stations */
#define OR_OPS_HODO_MATCH 30
/* one chi2_track term: the wire end points 6, the line's denominator 20,
 * the DCA numerator 14, sqrt and division 2, drift*sign - DCA 2, r*r/s/s and
 * the sum 4 */
#define OR_OPS_CHI2_HIT 48

#define OR_OPS_YZ_FIRST(n) ((n) * (OR_OPS_CALC_Y + OR_OPS_FIT_POINT) + OR_OPS_FIT_FIXED + OR_OPS_YZ_CUT1)
#define OR_OPS_YZ_SURVIVOR(n, nx)                                                                              \
    (((n) / 2) * OR_OPS_LR_PAIR + (n) * OR_OPS_LR_SINGLE + (n) * OR_OPS_FIT_POINT + OR_OPS_FIT_FIXED +         \
     OR_OPS_YZ_CUT2 + OR_OPS_PROP_MATCH + OR_OPS_HODO_MATCH + ((n) + (nx)) * OR_OPS_CHI2_HIT)

#endif /* OR_OPCOUNT_H */
