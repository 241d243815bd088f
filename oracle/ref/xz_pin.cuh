// xz_pin.cuh -- TEST INFRASTRUCTURE ONLY: the XZ stage's candidates computed
// by the reference's own __device__ helpers, compiled into the reference
// images through ref_kernels.cu (oracle/ref/build_ref.py).
//
// The reference's XZ kernel (OnlineReconstruction/reconstruction_kernels.cuh
// :182-855) cannot be run: its slot placement (:675-807) calls
// __syncthreads() in thread-dependent branches.  Everything before that
// placement is per thread and calls helpers:
//
//   make_hitpairs_in_station_bins  reconstruction_helper.cuh:368-460
//   calculate_xz_fy                reconstruction_helper.cuh:140-158
//   fit_2D_track / _drift          trackanalyticalminimizer.cuh:32-119
//   resolve_leftright_xhits        reconstruction_helper.cuh:808-872
//   resolve_single_leftright_xhits reconstruction_helper.cuh:875-892
//   match_track_XZ_to_hodo         reconstruction_helper.cuh:1090-1144
//
// xz_pin_kernel runs that per-thread part for each (event, reference thread
// t = 0..31) as one CUDA thread with no barrier, calling those helpers, and
// appends every candidate that passes all gates (the point where the kernel
// would place it in a tracklet slot) to the thread's output list, in the
// thread's order.  The loop structure, the bin split of the 32 threads
// (K:217-219), the prop-tube gate (K:577-640, inline code in the kernel) and
// the record layout are this file's own restatement; the arithmetic of every
// helper is the reference's compiled code.  Two departures, both at
// undefined behaviour of the reference:
//   - the per-thread hit scratch (K:378-396) gets a fifth entry holding a
//     plane id that pairs with nothing: the left/right walk reads the entry
//     past the hit count, which for four hits is past the reference's
//     four-entry arrays, and entries never written before are uninitialised
//     there (here: that plane id and zeros);
//   - the pair arrays hold MaxHitsProj_X + 1 pairs per bin, the last index
//     the pairing helper writes (the reference's hold MaxHitsProj_X, K:232).
#pragma once

namespace xzpin {
constexpr int NB = 7;                                        // bins per station and thread (K:202-205)
constexpr int PAIRS = NB * (globalconsts::MaxHitsProj_X + 1);
constexpr int REC = 32;                                      // floats per output record
constexpr int MAXH = 100;                                    // the pairing helper's hit flags (H:378-380)
constexpr short NOPLANE = -100;                              // a plane id no hit plane is adjacent to
// status bits per (event, thread)
constexpr int ST_BIN_OVERFLOW = 1;  // a bin of this thread holds more than MaxHitsProj_X pairs (K:359-375)
constexpr int ST_DOMAIN = 2;        // an x plane holds more hits than the helper's flags
constexpr int ST_OUT_FULL = 4;      // more accepted candidates than the output list holds
}  // namespace xzpin

// Output record r of (event e, thread t) at out[((e*32 + t)*cap + r)*REC]:
//   [0] binId = t + 32*i (K:446), [1] t, [2] number of hits, [3] x0, [4] tx,
//   [5] err_x0, [6] err_tx, [7] 0, then per hit n < 4 at 8 + 6n:
//   detector id, element id, x (calculate_xz_fy), drift, sign, tdc.
extern "C" __global__ void xz_pin_kernel(gEventHitCollections *hc, const gPlane *planes, const bool *skip,
                                         int n_events, float *out, int cap, int *nout, int *status) {
    using namespace xzpin;
    const long gt = (long)blockIdx.x * blockDim.x + threadIdx.x;
    if (gt >= (long)n_events * 32) return;
    const int e = (int)(gt / 32), t = (int)(gt % 32);
    nout[gt] = 0;
    status[gt] = 0;
    if (skip[e]) return;
    const short bin0_st2 = (short)((t / 8) * NB), bin0_st3 = (short)((t % 8 / 2) * NB);
    const int st3 = 3 + t % 2;
    short det[4];
    det[0] = (short)(globalconsts::detsuperid[2][0] * 2);
    det[1] = (short)(det[0] - 1);
    det[2] = (short)(globalconsts::detsuperid[st3][0] * 2);
    det[3] = (short)(det[2] - 1);
    int nh0, nh1, nh2, nh3;
    const gHits h0 = hc->hitschambers(e, det[0], nh0);
    const gHits h1 = hc->hitschambers(e, det[1], nh1);
    const gHits h2 = hc->hitschambers(e, det[2], nh2);
    const gHits h3 = hc->hitschambers(e, det[3], nh3);
    if (nh0 > MAXH || nh1 > MAXH || nh2 > MAXH || nh3 > MAXH) {
        status[gt] = ST_DOMAIN;
        return;
    }
    short flag1[MAXH], flag2[MAXH];
    int np2[NB], np3[NB];
    thrust::pair<int, int> pairs2[PAIRS], pairs3[PAIRS];
    make_hitpairs_in_station_bins(h0, nh0, h1, nh1, pairs2, np2, bin0_st2, NB, flag1, flag2, 2);
    make_hitpairs_in_station_bins(h2, nh2, h3, nh3, pairs3, np3, bin0_st3, NB, flag1, flag2, st3);
    for (int b = 0; b < NB; ++b)
        if (np2[b] > globalconsts::MaxHitsProj_X || np3[b] > globalconsts::MaxHitsProj_X) {
            status[gt] = ST_BIN_OVERFLOW;
            return;
        }
    // prop tubes and hodoscopes of the x view (K:302-354)
    const short dp1 = (short)(globalconsts::detsuperid[5][0] * 2), dp2 = (short)(globalconsts::detsuperid[6][0] * 2);
    int n_p11, n_p12, n_p21, n_p22;
    const gHits p11 = hc->hitsprop(e, dp1, n_p11), p12 = hc->hitsprop(e, dp1 - 1, n_p12);
    const gHits p21 = hc->hitsprop(e, dp2, n_p21), p22 = hc->hitsprop(e, dp2 - 1, n_p22);
    const float z_p11 = planes->z[dp1], z_p12 = planes->z[dp1 - 1];
    const float z_p21 = planes->z[dp2], z_p22 = planes->z[dp2 - 1];
    const float res[4] = {planes->resolution[det[0]], planes->resolution[det[1]], planes->resolution[det[2]],
                          planes->resolution[det[3]]};
    const gHits *hx[4] = {&h0, &h1, &h2, &h3};
    const thrust::pair<int, int> *pr[2] = {pairs2, pairs3};

    // per-thread hit scratch, kept across candidates as the reference keeps it
    short detID[5], elID[5], sign[5];
    float X[5], errX[5], Z[5], drift[5], tdc[5];
    for (int k = 0; k < 5; ++k) {
        detID[k] = NOPLANE;
        elID[k] = 0;
        sign[k] = 0;
        X[k] = errX[k] = Z[k] = drift[k] = tdc[k] = 0.f;
    }
    float A_[4], Ainv_[4], B_[2], Par[2], ParErr[2], chi2;
    int nrec = 0;
    float *dst = out + gt * (long)cap * REC;
    for (short i = 0; i < NB * NB; ++i) {
        const short bin2 = (short)(i % NB), bin3 = (short)((i - bin2) / NB);
        const int nx2 = np2[bin2], nx3 = np3[bin3];
        if (nx2 == 0 || nx3 == 0) continue;
        for (int c = 0; c < nx2 * nx3; ++c) {
            const int i_x2 = c % nx2, i_x3 = (c - i_x2) / nx2;
            const thrust::pair<int, int> p[2] = {pairs2[bin2 + NB * i_x2], pairs3[bin3 + NB * i_x3]};
            short nhits = 0, nhits2 = 0;
            for (int st = 0; st < 2; ++st) {
                for (int side = 0; side < 2; ++side) {
                    const int ih = side == 0 ? p[st].first : p[st].second;
                    if (ih < 0) continue;
                    const gHits &h = *hx[2 * st + side];
                    detID[nhits] = det[2 * st + side];
                    errX[nhits] = res[2 * st + side];
                    elID[nhits] = (short)h.chan(ih);
                    tdc[nhits] = h.tdc(ih);
                    drift[nhits] = h.drift(ih);
                    sign[nhits] = 0;
                    calculate_xz_fy(detID[nhits], elID[nhits], drift[nhits], sign[nhits], 0, 0, planes, X[nhits],
                                    Z[nhits]);
                    ++nhits;
                }
                if (st == 0) {
                    nhits2 = nhits;
                    if (nhits2 == 0) break;
                }
            }
            if (nhits2 == 0 || nhits == nhits2) continue;  // K:510, K:544
            fit_2D_track(nhits, X, Z, errX, A_, Ainv_, B_, Par, ParErr, chi2);
            float x0 = Par[0], tx = Par[1], errx0 = ParErr[0], errtx = ParErr[1];
            if (fabs(x0) > X0_MAX + 2 * errx0 || fabs(tx) > TX_MAX + 2 * errtx) continue;
            resolve_leftright_xhits(x0, tx, errx0, errtx, nhits, detID, X, drift, sign, planes->z, 150.);
            resolve_single_leftright_xhits(x0, tx, nhits, detID, X, sign, planes->z);
            fit_2D_track_drift(nhits, X, drift, sign, Z, errX, A_, Ainv_, B_, Par, ParErr, chi2);
            x0 = Par[0];
            tx = Par[1];
            errx0 = ParErr[0];
            errtx = ParErr[1];
            if (fabs(x0) > X0_MAX || fabs(tx) > TX_MAX) continue;
            // prop tubes: a hit within 5.08 cm in P1 (first plane, else the
            // second) and within 7.62 cm in P2, counted per station
            short nprop = 0;
            bool found = false;
            for (int n = 0; n < n_p11 && !found; ++n) found = fabs(p11.pos(n) - (tx * z_p11 + x0)) < 5.08f;
            for (int n = 0; n < n_p12 && !found; ++n) found = fabs(p12.pos(n) - (tx * z_p12 + x0)) < 5.08f;
            nprop += found;
            found = false;
            for (int n = 0; n < n_p21 && !found; ++n) found = fabs(p21.pos(n) - (tx * z_p21 + x0)) < 7.62f;
            for (int n = 0; n < n_p22 && !found; ++n) found = fabs(p22.pos(n) - (tx * z_p22 + x0)) < 7.62f;
            nprop += found;
            if (nprop < selection::NpropXYhitsMin) continue;
            bool hodo = true;
            for (int s = 1; s < 4 && hodo; ++s) {
                int nh_a, nh_b;
                const gHits ha = hc->hitshodos(e, globalconsts::hodoplanesx[s][0], nh_a);
                const gHits hb = hc->hitshodos(e, globalconsts::hodoplanesx[s][1], nh_b);
                hodo = match_track_XZ_to_hodo(s, globalconsts::hodoplanesx[s][0], nh_a, ha, x0, tx, errx0, errtx,
                                              planes->z) ||
                       match_track_XZ_to_hodo(s, globalconsts::hodoplanesx[s][1], nh_b, hb, x0, tx, errx0, errtx,
                                              planes->z);
            }
            if (!hodo) continue;
            if (nrec >= cap) {
                status[gt] |= ST_OUT_FULL;
                continue;
            }
            float *r = dst + (long)nrec * REC;
            r[0] = (float)(t + 32 * i);
            r[1] = (float)t;
            r[2] = (float)nhits;
            r[3] = x0;
            r[4] = tx;
            r[5] = errx0;
            r[6] = errtx;
            r[7] = 0.f;
            for (int n = 0; n < 4; ++n) {
                const bool on = n < nhits;
                r[8 + 6 * n] = on ? (float)detID[n] : 0.f;
                r[9 + 6 * n] = on ? (float)elID[n] : 0.f;
                r[10 + 6 * n] = on ? X[n] : 0.f;
                r[11 + 6 * n] = on ? drift[n] : 0.f;
                r[12 + 6 * n] = on ? (float)sign[n] : 0.f;
                r[13 + 6 * n] = on ? tdc[n] : 0.f;
            }
            ++nrec;
        }
    }
    nout[gt] = nrec;
}
