// global_kernel.cu -- global tracking across KMag (station-1 extension).
//
// Replaces gKernel_Global_tracking<<<N,32>>> (OnlineReconstruction/
// reconstruction_kernels.cuh:1841-2534).
//
// Per YZ track (stationID >= 5) the reference finds station-1 x/u/v hit
// pairs in sagitta windows (reconstruction_helper.cuh:556-613), then for
// each x1 pair fits the x hits plus the KMag bend point, derives charge and
// 1/p (H:652-691), and for each (u1, v1) combination fits y with the
// station-2/3 u/v hits, resolves left/right, and keeps the best chi2.
// State carried by the reference, reproduced here:
//   - y0/ty are overwritten by every (u1,v1) fit and feed the next x1 pair's
//     x positions (K:2120, K:2370-2377);
//   - on the x' hit alone, the walk pairs it with the first u1 hit (planes
//     3/2) and re-sets its sign whenever that resolution succeeds;
//   - the scratch entry past the hit count (x part and uv part of the walk).
// One warp per event; slots, tracks and x1 pairs in order; (u1, v1)
// combinations 32 at a time with ballot/shuffle scans for that state.
#include "window_pairs.cuh"

namespace orgpu {

constexpr int GL_PAIRCAP = 128;
constexpr int GL_NST = 7;  // scratch entries tracked for stale reads: 0..6


struct GlWarp {
    HitPlane hc[6];  // station-1 plane views of the current event, the same for every lane
    short dl[6];
    short2 pairs[3][GL_PAIRCAP];  // x1, u1, v1
    WindowScratch W;
    // station-2/3 hits of the current track
    short s_det[12], s_chan[12], s_sign[12];
    float s_drift[12], s_res[12];
    float Y[12], eY[12], Zy[12];
    // the current track's (u1, v1) y fit by plane set (gl_tab_entry)
    float tab[9][8];
    // best
    float b_chi2, b_ty, b_y0, b_invp, b_ety, b_ey0, b_einvp, b_charge;
    int b_n;
    float b_det[6], b_el[6], b_pos[6], b_drift[6], b_sign[6], b_tdc[6], b_res[18];
};

// The y fit of a (u1, v1) combination (K:2368-2379) adds the track's
// station-2/3 y hits and then the accepted u1 u1' v1 v1' hits, each with its
// plane's weight (calculate_y_uvhit's error, a plane constant) and z: its
// normal matrix, inverse and errors depend only on which station-1 planes
// gave a hit.  Entry (gu - 1) * 3 + gv - 1 (plane bits of the u1 and v1
// groups, 1..3) holds Fit2::solve's inverse A^-1 (4), the 2-sigma bounds of
// the first cut Y0_MAX + 2 err_y0, TY_MAX + 2 err_ty, and err_y0, err_ty --
// computed as Fit2 accumulates (the station-2/3 hits first, the station-1
// planes in attempt order), so a combination needs only its right-hand side.
__device__ __forceinline__ void gl_tab_entry(const float *eY, const float *Zy, int nyh, int gu, int gv,
                                             const short *dl, const or_plane_t &P, float *out) {
    Fit2 f;
#pragma unroll 1
    for (int k = 0; k < nyh; ++k) f.add(0.f, Zy[k], eY[k]);
    const int lists[4] = {2, 3, 4, 5};
#pragma unroll
    for (int a = 0; a < 4; ++a) {
        if (!((a < 2 ? gu >> a : gv >> (a - 2)) & 1)) continue;
        const int d = dl[lists[a]];
        f.add(0.f, P.z[d], P.resolution[d] * fabsf(P.deltapy[d] / P.deltapx[d]));
    }
    const float A[4] = {f.A0, f.A1, f.A2, f.A3};
    float Ai[4];
    matinv_2x2(A, Ai);
    const float e0 = sqrtf(fabsf(Ai[0])), e1 = sqrtf(fabsf(Ai[3]));
    out[0] = Ai[0];
    out[1] = Ai[1];
    out[2] = Ai[2];
    out[3] = Ai[3];
    out[4] = Y0_MAX + 2 * e0;
    out[5] = TY_MAX + 2 * e1;
    out[6] = e0;
    out[7] = e1;
}

struct GHit {
    short det, el, sign;
    float pos, drift, tdc;
};

struct Stale {
    short det;
    float pos, drift;
};

// SagittaRatioInStation1, H:556-613
static __device__ void sagitta_st1(float x0, float tx, float y0, float ty, int detid_lasthit, float *pos_exp, float *window,
                            const or_plane_t &P) {
    const float z_st3 = P.z[detid_lasthit];
    const float x_st3 = x0 + tx * z_st3;
    const float y_st3 = y0 + ty * z_st3;
#pragma unroll 1
    for (int i = 0; i < 3; i++) {
        const short detid = (short)(2 * i + 2);
        const short idx = c_planetype[detid / 2 - 1];
        const short detid_2 = (short)(c_detsuperid[2][idx] * 2);
        const float pos_st3 = x_st3 * P.costheta[detid_2] + y_st3 * P.sintheta[detid_2];
        const float z_st1 = P.z[detid];
        const float z_st2 = P.z[detid_2];
        const float x_st2 = x0 + tx * z_st2;
        const float y_st2 = y0 + ty * z_st2;
        const float pos_st2 = x_st2 * P.costheta[detid_2] + y_st2 * P.sintheta[detid_2];
        const float s2_target = pos_st2 - pos_st3 * (z_st2 - Z_TARGET) / (z_st3 - Z_TARGET);
        const float s2_dump = pos_st2 - pos_st3 * (z_st2 - Z_DUMP) / (z_st3 - Z_DUMP);
        const float pe_t = SAGITTA_TARGET_CENTER * s2_target + pos_st3 * (z_st1 - Z_TARGET) / (z_st3 - Z_TARGET);
        const float pe_d = SAGITTA_DUMP_CENTER * s2_dump + pos_st3 * (z_st1 - Z_DUMP) / (z_st3 - Z_DUMP);
        const float win_t = fabsf(s2_target * SAGITTA_TARGET_WIDTH);
        const float win_d = fabsf(s2_dump * SAGITTA_DUMP_WIDTH);
        const float p_min = fminf(pe_t - win_t, pe_d - win_d);
        const float p_max = fmaxf(pe_t + win_t, pe_d + win_d);
        pos_exp[idx] = (float)(0.5 * (double)(p_max + p_min));
        window[idx] = (float)(0.5 * (double)(p_max - p_min));
    }
}

// Work units are (event, group of GL_CHUNK slots), taken from a device
// counter: slots are independent in the reference (one thread each, state
// kept per thread), and the cost per event is very uneven, so warps that
// finish early keep taking units instead of idling behind a heavy event.
#ifndef OR_GL_CHUNK
#define OR_GL_CHUNK 4
#endif
constexpr int GL_CHUNK = OR_GL_CHUNK;

// The survivor work of the (u1,v1) loop -- left/right walk and chi2 --
// kept out of line (one copy each) so that the loop's instructions stay
// resident in the instruction cache.

// resolve_leftright_newhits over the x + uv hits (H:714-780), with the
// scratch entry past the end, then the singles (H:785-804)
__device__ __noinline__ void gl_walk(GHit *h, int nall, const Stale &st, float xs0, float xst, float yc, float tyc,
                                     float ex0s, float etxs, float eyc, float etyc, const or_plane_t &P) {
#pragma unroll 1
    for (int i = 0; i < nall;) {
        const int j = i + 1;
        const short di = h[i].det;
        const short dj = j < nall ? h[j].det : st.det;
        if (abs(di - dj) != 1) {
            i += 1;
            continue;
        }
        const short sj = j < nall ? h[j].sign : (short)0;
        if (h[i].sign * sj == 0) {
            const float pj = j < nall ? h[j].pos : st.pos;
            const float drj = j < nall ? h[j].drift : st.drift;
            const int k = lr_pair_newhits(xs0, xst, yc, tyc, ex0s, etxs, eyc, etyc, di, dj, h[i].pos, h[i].drift, pj,
                                          drj, P, 150.f);
            if (k >= 0) {
                h[i].sign = c_lrpossibility[k][0];
                if (j < nall) h[j].sign = c_lrpossibility[k][1];
            }
        }
        i += 2;
    }
#pragma unroll 1
    for (int k = 0; k < nall; ++k)
        if (!h[k].sign) h[k].sign = single_sign_newhits(xs0, xst, yc, tyc, h[k].det, h[k].pos, P);
}

// chi2 over the station-2/3 hits (H:1149-1180) plus chi2_track over the
// station-1 hits (K:2449-2461); residuals into rst / rs1
__device__ __noinline__ float gl_chi2(const GlWarp &S, int nst, const GHit *h, int nall, const or_plane_t &P, float x0,
                                      float tx, float xs0, float xst, float yc, float tyc, float *rst, float *rs1) {
    float chi2 = 0.f;
#pragma unroll 1
    for (int m = 0; m < nst && m < 12; ++m) {
        const short d = S.s_det[m];
        const float r = residual_line(x_bep(d, S.s_chan[m], P), y_bep(d, S.s_chan[m], P), z_bep(d, S.s_chan[m], P),
                                      P.deltapx[d], P.deltapy[d], P.deltapz[d], S.s_drift[m], S.s_sign[m], x0, yc, tx,
                                      tyc);
        rst[m] = r;
        chi2 += r * r / (S.s_res[m] * S.s_res[m]);
    }
    float c1 = 0.f;
#pragma unroll 1
    for (int k = 0; k < nall; ++k) {
        const short d = h[k].det;
        const float r = residual_line(x_bep(d, h[k].el, P), y_bep(d, h[k].el, P), z_bep(d, h[k].el, P), P.deltapx[d],
                                      P.deltapy[d], P.deltapz[d], h[k].drift, h[k].sign, xs0, yc, xst, tyc);
        rs1[k] = r;
        c1 += r * r / P.resolution[d] / P.resolution[d];
    }
    return chi2 + c1;
}

template <int W>
__global__ void __launch_bounds__(W * 32)
    global_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
                  const uint8_t *__restrict__ toomany, int n_events, uint32_t *__restrict__ errw,
                  unsigned long long *__restrict__ sched) {
    extern __shared__ __align__(16) unsigned char gl_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(gl_smem);
    GlWarp *warps = reinterpret_cast<GlWarp *>(gl_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    GlWarp &S = warps[w];
    // station-1 planes x x' u u' v v' (K:1880-1923, E1039 chamber ids)
    if (lane == 0) {
        const short dl0[6] = {4, 3, 2, 1, 6, 5};
#pragma unroll
        for (int k = 0; k < 6; ++k) S.dl[k] = dl0[k];
    }
    __syncwarp();
    const short *dl = S.dl;

    const unsigned long long nunits = (unsigned long long)n_events * (OR_NSLOTS / GL_CHUNK);
    for (;;) {
        unsigned long long u = 0;
        if (lane == 0) u = atomicAdd(sched, 1ull);
        u = __shfl_sync(0xffffffffu, u, 0);
        if (u >= nunits) break;
        const long e = (long)(u / (OR_NSLOTS / GL_CHUNK));
        const int slot0 = (int)(u % (OR_NSLOTS / GL_CHUNK)) * GL_CHUNK;
        if (toomany[e]) continue;
        HitPlane *hc = S.hc;
        __syncwarp();  // every lane is done with the previous event's views
        if (lane == 0) {
#pragma unroll 1
            for (int k = 0; k < 6; ++k) hc[k] = hits_of(hv, e, dl[k]);
        }
        __syncwarp();
#pragma unroll 1
        for (int slot = slot0; slot < slot0 + GL_CHUNK; ++slot) {
            const int ntr = min((int)tv.ntracks[e * OR_NSLOTS + slot], OR_SLOTCAP);
            if (ntr == 0) continue;
            Stale stc[GL_NST];
#pragma unroll 1
            for (int k = 0; k < GL_NST; ++k) stc[k] = Stale{DET_SENTINEL, 0.f, 0.f};
#pragma unroll 1
            for (int it = 0; it < ntr; ++it) {
                float *T = trk_rec(tv, e, slot, it);
                const short nst = (short)min((int)T[OR_TRK_NHITS], 12);  // YZ tracks carry <= 12 hits
                if (T[OR_TRK_STID] < 5) continue;  // K:2053
                const float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], ex0 = T[OR_TRK_ERR_X0], etx = T[OR_TRK_ERR_TX];
                float y0 = T[OR_TRK_Y0], ty = T[OR_TRK_TY];
                // get_lasthitdetid (reconstruction_classes.cuh:500-515)
                short dmax = 1;
                float zmax = -10000.f;
#pragma unroll 1
                for (short k = 0; k < nst; ++k) {
                    const short d = (short)T[OR_TRK_HIT_DETID + k];
                    if (d > 0 && P.z[d] > zmax) {
                        dmax = d;
                        zmax = P.z[d];
                    }
                }
                float pexp[3], win[3];
                sagitta_st1(x0, tx, y0, ty, dmax, pexp, win, P);
                int np[3];
                bool overcap = false;
#pragma unroll 1
                for (int q = 0; q < 3; ++q) {
                    const float spacing = c_spacingplane[c_detsuperid[0][q]];
                    np[q] = window_pairs(hc[2 * q], dl[2 * q], hc[2 * q + 1], dl[2 * q + 1], spacing,
                                         pexp[q] - win[q] * 1.0f, pexp[q] + win[q] * 1.0f, P, S.pairs[q], GL_PAIRCAP,
                                         S.W);
                    overcap |= np[q] > GL_PAIRCAP;
                }
                if (overcap) {
                    if (lane == 0) atomicOr(errw, ERRW_CAPACITY);
                    continue;
                }
                const int nx1 = np[0], nu1 = np[1], nv1 = np[2];
                if (nx1 == 0 || nu1 == 0 || nv1 == 0) continue;
                // station-2/3 hits and their y (K:2086-2102)
                int nyh = 0;
#pragma unroll 1
                for (int k = 0; k < nst && k < 12; ++k) {
                    const short d = (short)T[OR_TRK_HIT_DETID + k];
                    const float dr = T[OR_TRK_HIT_DRIFT + k];
                    const short sg = (short)T[OR_TRK_HIT_SIGN + k];
                    if (lane == 0) {
                        S.s_det[k] = d;
                        S.s_chan[k] = (short)T[OR_TRK_HIT_CHAN + k];
                        S.s_drift[k] = dr;
                        S.s_sign[k] = sg;
                        S.s_res[k] = P.resolution[d];
                    }
                    if ((double)P.costheta[d] > 0.99) continue;
                    float yy, ey;
                    if (calculate_y_uvhit((int)T[OR_TRK_HIT_DETID + k], (int)T[OR_TRK_HIT_CHAN + k], dr, sg, x0, tx, P,
                                          yy, ey)) {
                        if (lane == 0) {
                            S.Y[nyh] = yy;
                            S.eY[nyh] = ey;
                            S.Zy[nyh] = P.z[d];
                        }
                        ++nyh;
                    }
                }
                __syncwarp();
                // the y fit's station-1 plane sets, one per lane, and the
                // right-hand side of the station-2/3 hits (Fit2::add order)
                if (lane < 9) gl_tab_entry(S.eY, S.Zy, nyh, lane / 3 + 1, lane % 3 + 1, dl, P, S.tab[lane]);
                float bs0 = 0.f, bs1 = 0.f;
#pragma unroll 1
                for (int k = 0; k < nyh; ++k) {
                    bs0 += S.eY[k] * S.Y[k];
                    bs1 += S.eY[k] * S.Y[k] * S.Zy[k];
                }
                __syncwarp();
                float chi2min = 10000.1f;
                bool update = false;
                const int C = nu1 * nv1;
#pragma unroll 1
                for (int ix = 0; ix < nx1; ++ix) {
                    // x hits (K:2108-2159), uniform over the warp
                    const short2 px = S.pairs[0][ix];
                    GHit xh[2];
                    float X[3], eX[3], Zx[3];
                    int nhx = 0;
#pragma unroll 1
                    for (int wsel = 0; wsel < 2; ++wsel) {
                        const int hidx = wsel == 0 ? px.x : px.y;
                        if (hidx < 0) continue;
                        GHit &g = xh[nhx];
                        g.det = dl[wsel];
                        g.pos = hc[wsel].pos(hidx);
                        g.el = (short)hc[wsel].chan(hidx);
                        g.tdc = hc[wsel].tdc(hidx);
                        g.sign = 0;
                        g.drift = hc[wsel].drift(hidx);
                        eX[nhx] = P.resolution[dl[wsel]];
                        calculate_xz_fy(g.det, g.el, g.drift, 0, y0, ty, P, X[nhx], Zx[nhx]);
                        ++nhx;
                    }
#pragma unroll 1
                    for (int k = 0; k < nhx; ++k) stc[k] = Stale{xh[k].det, xh[k].pos, xh[k].drift};
                    X[nhx] = x0 + tx * Z_KMAG_BEND;  // K:2163-2165
                    eX[nhx] = ex0 + etx * Z_KMAG_BEND;
                    Zx[nhx] = Z_KMAG_BEND;
                    float xs0, xst, e0, e1;
                    {
                        Fit2 f;
#pragma unroll 1
                        for (int k = 0; k <= nhx; ++k) f.add(X[k], Zx[k], eX[k]);
                        f.solve(xs0, xst, e0, e1);
                    }
                    float ex0s = xs0, etxs = xst;  // K:2175-2176 as written
                    // resolve_leftright_xhits (H:820-871); the entry past the
                    // x hits holds the KMag point in X and stale det/drift
#pragma unroll 1
                    for (int n = 0; n < nhx;) {
                        const int j = n + 1;
                        const short di = xh[n].det;
                        const short dj = j < nhx ? xh[j].det : stc[j].det;
                        if (abs(di - dj) != 1) {
                            n += 1;
                            continue;
                        }
                        const float drj = j < nhx ? xh[j].drift : stc[j].drift;
                        const int k = lr_pair_xhits(xs0, xst, ex0s, etxs, di, dj, X[n], xh[n].drift, X[j], drj, P.z,
                                                    150.f);
                        if (k >= 0) {
                            xh[n].sign = c_lrpossibility[k][0];
                            if (j < nhx) xh[j].sign = c_lrpossibility[k][1];
                        }
                        n += 2;
                    }
#pragma unroll 1
                    for (int k = 0; k < nhx; ++k)
                        if (!xh[k].sign) xh[k].sign = single_sign_xhits(xs0, xst, xh[k].det, X[k], P.z);
#pragma unroll 1
                    for (int k = 0; k < nhx; ++k) X[k] += (float)xh[k].sign * xh[k].drift;
                    {
                        Fit2 f;
#pragma unroll 1
                        for (int k = 0; k <= nhx; ++k) f.add(X[k], Zx[k], eX[k]);
                        f.solve(xs0, xst, e0, e1);
                    }
                    ex0s = xs0;
                    etxs = xst;
                    const short charge = calculate_charge(tx, x0);  // K:2198-2203
                    const float invP = (xst - tx) * (float)charge / PT_KICK_KMAG;
                    const float einvP = (etx - etx) / PT_KICK_KMAG;
                    if (invP > INVP_MAX + einvP || invP < INVP_MIN - einvP) continue;
                    // carried across (u1,v1) chunks
                    bool has_y = false;
                    float ny0 = 0.f, nty = 0.f;
                    bool xcarry = false;
                    short xcarry_v = 0;
#pragma unroll 1
                    for (int base = 0; base < C; base += 32) {
                        const int c = base + lane;
                        const bool valid = c < C;
                        GHit h[6];
#pragma unroll 1
                        for (int k = 0; k < nhx; ++k) h[k] = xh[k];
                        float b0 = bs0, b1 = bs1;  // the y fit's right-hand side
                        int nuv = 0, nhu = 0, gb = 0;  // gb: plane bits u1 u1' v1 v1' of the accepted hits
                        // scratch entries this combination writes: (list << 12 | hit index)
                        // codes, 16 bits each, entries 0-3 and 4-6
                        unsigned long long own_lo = 0ull, own_hi = 0ull;
                        unsigned wmask = 0u;
                        bool reached = false, pass1 = false;
                        float yc = 0.f, tyc = 0.f, eyc = 0.f, etyc = 0.f;
                        if (valid) {
                            const int iu = c % nu1, iv = c / nu1;
                            const short2 pu = S.pairs[1][iu], pv = S.pairs[2][iv];
                            auto attempt = [&](int lk, int hidx) {  // K:2221-2288
                                const int a = nhx + nuv;
                                GHit &u = h[a];
                                u.det = dl[lk];
                                u.el = (short)hc[lk].chan(hidx);
                                u.tdc = hc[lk].tdc(hidx);
                                u.sign = 0;
                                u.drift = hc[lk].drift(hidx);
                                u.pos = hc[lk].pos(hidx);
                                if (a < GL_NST) {
                                    const unsigned long long code = (unsigned long long)((lk << 12) | hidx);
                                    if (a < 4) own_lo = (own_lo & ~(0xFFFFull << (16 * a))) | (code << (16 * a));
                                    else own_hi = (own_hi & ~(0xFFFFull << (16 * (a - 4)))) | (code << (16 * (a - 4)));
                                    wmask |= 1u << a;
                                }
                                float yy, ey;
                                if (calculate_y_uvhit(u.det, u.el, u.drift, 0, xs0, xst, P, yy, ey)) {
                                    b0 += ey * yy;  // Fit2::add(yy, z, ey)
                                    b1 += ey * yy * P.z[dl[lk]];
                                    gb |= 1 << (lk - 2);
                                    ++nuv;
                                }
                            };
                            // u1, u1', then v1, v1' if the u1 group gave a hit, as one loop body
                            const unsigned long long codes =
                                (unsigned long long)(pu.x >= 0 ? (2 << 12) | pu.x : 0xFFFF) |
                                ((unsigned long long)(pu.y >= 0 ? (3 << 12) | pu.y : 0xFFFF) << 16) |
                                ((unsigned long long)(pv.x >= 0 ? (4 << 12) | pv.x : 0xFFFF) << 32) |
                                ((unsigned long long)(pv.y >= 0 ? (5 << 12) | pv.y : 0xFFFF) << 48);
#pragma unroll 1
                            for (int q = 0; q < 4; ++q) {
                                if (q == 2) {
                                    nhu = nuv;
                                    if (nhu == 0) break;
                                }
                                const int code = (int)((codes >> (16 * q)) & 0xFFFFull);
                                if (code != 0xFFFF) attempt(code >> 12, code & 0xFFF);
                            }
                            reached = nhu > 0 && nuv > nhu;
                            if (reached) {  // K:2368-2379, Fit2::solve with the plane set's inverse
                                const float *te = S.tab[((gb & 3) - 1) * 3 + (gb >> 2) - 1];
                                yc = 0.0f;
                                yc += te[0] * b0;
                                yc += te[1] * b1;
                                tyc = 0.0f;
                                tyc += te[2] * b0;
                                tyc += te[3] * b1;
                                eyc = te[6];
                                etyc = te[7];
                                pass1 = !(fabsf(yc) > te[4] || fabsf(tyc) > te[5]);
                            }
                        }
                        const int nall = nhx + nuv;
                        // scratch entry past the hit count
                        Stale st{DET_SENTINEL, 0.f, 0.f};
                        int st_code = -1;
                        {
                            const unsigned lt = lanemask_lt();
                            auto decode = [&](int code) {
                                const int lk = code >> 12, hidx = code & 0xFFF;
                                return Stale{dl[lk], hc[lk].pos(hidx), hc[lk].drift(hidx)};
                            };
#pragma unroll 1
                            for (int k = 0; k < GL_NST; ++k) {
                                const bool mine = (wmask >> k) & 1u;
                                const int code = (int)(((k < 4 ? own_lo : own_hi) >> (16 * (k & 3))) & 0xFFFFull);
                                const unsigned m = __ballot_sync(0xffffffffu, mine);
                                const int src = last_lane(m & lt);
                                const int sc = __shfl_sync(0xffffffffu, code, src < 0 ? 0 : src);
                                if (nall == k) {
                                    if (mine) st_code = code;
                                    else if (src >= 0) st_code = sc;
                                    else st = stc[k];
                                }
                                const int lw = last_lane(m);
                                if (lw >= 0) stc[k] = decode(__shfl_sync(0xffffffffu, code, lw));
                            }
                            if (pass1 && st_code >= 0) st = decode(st_code);
                        }
                        // y0/ty of the last combination that reached the fit
                        {
                            const unsigned rm = __ballot_sync(0xffffffffu, reached);
                            const int rl = last_lane(rm);
                            const float vy = __shfl_sync(0xffffffffu, yc, rl < 0 ? 0 : rl);
                            const float vt = __shfl_sync(0xffffffffu, tyc, rl < 0 ? 0 : rl);
                            if (rl >= 0) {
                                has_y = true;
                                ny0 = vy;
                                nty = vt;
                            }
                        }
                        // x' hit alone, paired with the first u1 hit (planes 3, 2)
                        bool xok = false;
                        short xval = 0;
                        const bool cross = pass1 && nhx == 1 && h[0].det == 3 && h[1].det == 2;
                        if (cross) {
                            const int k = lr_pair_newhits_ool(xs0, xst, yc, tyc, ex0s, etxs, eyc, etyc, h[0].det,
                                                              h[1].det, h[0].pos, h[0].drift, h[1].pos, h[1].drift, P,
                                                              150.f);
                            if (k >= 0) {
                                xok = true;
                                xval = c_lrpossibility[k][0];
                            }
                        }
                        const unsigned xm = __ballot_sync(0xffffffffu, xok);
                        const int xs = last_lane(xm & lanemask_lt());
                        const short xprev = (short)__shfl_sync(0xffffffffu, (int)xval, xs < 0 ? 0 : xs);
                        float chi2 = 0.f;
                        float rst[12], rs1[6];
                        bool pass = false;
                        if (pass1) {
                            if (nhx == 1 && h[0].det == 3) {
                                if (xs >= 0) h[0].sign = xprev;
                                else if (xcarry) h[0].sign = xcarry_v;
                            }
                            gl_walk(h, nall, st, xs0, xst, yc, tyc, ex0s, etxs, eyc, etyc, P);
                            pass = !(fabsf(yc) > Y0_MAX || fabsf(tyc) > TY_MAX);  // K:2410
                            if (pass) {  // K:2449-2461
                                chi2 = gl_chi2(S, nst, h, nall, P, x0, tx, xs0, xst, yc, tyc, rst, rs1);
                                pass = !(chi2 > 10000.f);
                            }
                        }
                        // carry of the x' sign to the next chunk
                        {
                            const int xl = last_lane(xm);
                            const short nx = (short)__shfl_sync(0xffffffffu, (int)xval, xl < 0 ? 0 : xl);
                            if (xl >= 0) {
                                xcarry = true;
                                xcarry_v = nx;
                            }
                        }
                        // best chi2, strict < in combination order (K:2470)
                        const bool elig = pass && chi2 < chi2min;
                        const unsigned key = elig ? __float_as_uint(chi2) : 0xffffffffu;
                        const unsigned kmin = __reduce_min_sync(0xffffffffu, key);
                        if (kmin != 0xffffffffu) {
                            const int winl = __ffs(__ballot_sync(0xffffffffu, key == kmin)) - 1;
                            if (lane == winl) {
                                S.b_n = nall;
                                S.b_chi2 = chi2;
                                S.b_ty = tyc;
                                S.b_y0 = yc;
                                S.b_invp = invP;
                                S.b_ety = etyc;
                                S.b_ey0 = eyc;
                                S.b_einvp = einvP;
                                S.b_charge = (float)charge;
#pragma unroll 1
                                for (int m = 0; m < nst && m < 12; ++m) S.b_res[m] = rst[m];
#pragma unroll 1
                                for (int k = 0; k < nall; ++k) {
                                    S.b_det[k] = h[k].det;
                                    S.b_el[k] = h[k].el;
                                    S.b_pos[k] = h[k].pos;
                                    S.b_drift[k] = h[k].drift;
                                    S.b_sign[k] = h[k].sign;
                                    S.b_tdc[k] = h[k].tdc;
                                    S.b_res[nst + k] = rs1[k];
                                }
                            }
                            chi2min = __uint_as_float(kmin);
                            update = true;
                            __syncwarp();
                        }
                    }
                    if (has_y) {
                        y0 = ny0;
                        ty = nty;
                    }
                }
                if (update) {  // K:2504-2528
                    __syncwarp();
                    const int n1 = S.b_n;
                    if (lane == 0) {
                        T[OR_TRK_STID] = 6.f;
                        T[OR_TRK_NHITS] = (float)nst + (float)n1;
                        T[OR_TRK_CHI2] = S.b_chi2;
                        T[OR_TRK_TY] = S.b_ty;
                        T[OR_TRK_Y0] = S.b_y0;
                        T[OR_TRK_INVP] = S.b_invp;
                        T[OR_TRK_ERR_TY] = S.b_ety;
                        T[OR_TRK_ERR_Y0] = S.b_ey0;
                        T[OR_TRK_ERR_INVP] = S.b_einvp;
                        T[OR_TRK_CHARGE] = S.b_charge;
                    }
                    if (lane < nst && lane < 12) T[OR_TRK_HIT_RESID + lane] = S.b_res[lane];
                    if (lane < n1) {
                        const int n = lane;
                        T[OR_TRK_HIT_DETID + nst + n] = S.b_det[n];
                        T[OR_TRK_HIT_CHAN + nst + n] = S.b_el[n];
                        T[OR_TRK_HIT_POS + nst + n] = S.b_pos[n];
                        T[OR_TRK_HIT_DRIFT + nst + n] = S.b_drift[n];
                        T[OR_TRK_HIT_SIGN + nst + n] = S.b_sign[n];
                        T[OR_TRK_HIT_TDC + nst + n] = S.b_tdc[n];
                        T[OR_TRK_HIT_RESID + nst + n] = S.b_res[nst + n];
                    }
                }
                __syncwarp();
            }
        }
    }
}

size_t global_smem_bytes(int warps) {
    return ((sizeof(or_plane_t) + 15) & ~size_t(15)) + sizeof(GlWarp) * (size_t)warps;
}

template <int W>
static cudaError_t global_launch(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv,
                                 const uint8_t *toomany, int n_events, uint32_t *errw, unsigned long long *sched,
                                 cudaStream_t stream, int sm_count) {
    const size_t smem = global_smem_bytes(W);
    cudaError_t err = smem_attr_once((const void *)global_kernel<W>, (int)smem);
    if (err != cudaSuccess) return err;
    if ((err = cudaMemsetAsync(sched, 0, sizeof(unsigned long long), stream)) != cudaSuccess) return err;
    long blocks = ((long)n_events * (OR_NSLOTS / GL_CHUNK) + W - 1) / W;
    const long cap = (long)sm_count * (32 / W > 0 ? 32 / W : 1);
    if (blocks > cap) blocks = cap;
    global_kernel<W><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, toomany, n_events, errw, sched);
    return cudaGetLastError();
}

// `warps` = work units (event, 8 slots) in flight per CTA: 1, 2, 4, 8 or 16
cudaError_t launch_global(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                          int n_events, uint32_t *errw, unsigned long long *sched, cudaStream_t stream,
                          int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return global_launch<1>(d_plane, hv, tv, toomany, n_events, errw, sched, stream, sm_count);
    case 2: return global_launch<2>(d_plane, hv, tv, toomany, n_events, errw, sched, stream, sm_count);
    case 8: return global_launch<8>(d_plane, hv, tv, toomany, n_events, errw, sched, stream, sm_count);
    case 16: return global_launch<16>(d_plane, hv, tv, toomany, n_events, errw, sched, stream, sm_count);
    default: return global_launch<4>(d_plane, hv, tv, toomany, n_events, errw, sched, stream, sm_count);
    }
}

}  // namespace orgpu
