// yz_kernel.cu -- YZ extension of the XZ tracklets with U/V hits.
//
// Replaces gKernel_YZ_tracking<<<N,32>>> (OnlineReconstruction/
// reconstruction_kernels.cuh:864-1832).
//
// The reference gives each of its 32 threads one tracklet slot and, for every
// tracklet in it, loops u3 x v3 (outer) and u2 x v2 (inner) hit pairs
// sequentially, keeping the best chi2 (K:1320-1825).  Two pieces of state
// make that loop sequential:
//   - the station-3 hit signs chosen by the left/right resolution survive
//     from one inner iteration to the next: they are fixed by the first
//     combination of a (u3,v3) iteration that passes the first y cut, and on
//     station 3+ the last v3' hit can pair with the first u2 hit
//     (planes 19/18), whose resolution re-sets that sign whenever it
//     succeeds (H:714-780);
//   - the walk reads the scratch entry just past the hit count
//     (H:725-735), which holds the last hit load attempted at that index.
// Here lanes evaluate 32 (u3,v3,u2,v2) combinations at a time in the
// reference order and recover both pieces of state with ballot/shuffle
// scans carried across chunks, so the result equals the sequential loop.
// One warp per event walks the 32 slots and their tracklets in order.
#include "window_pairs.cuh"

namespace orgpu {

constexpr int YZ_WARPS = 4;
constexpr int YZ_PAIRCAP = 128;

struct YzWarp {
    short2 pairs[4][YZ_PAIRCAP];  // u2, v2, u3, v3
    WindowScratch W;
    float xdd[4], xres[4], xp1x[4], xp1y[4], xp1z[4], xdpx[4], xdpy[4], xdpz[4];
    short xhs[4];
    float b_chi2, b_ty, b_y0, b_ety, b_ey0;
    int b_nuv;
    float b_det[8], b_el[8], b_pos[8], b_drift[8], b_sign[8], b_tdc[8], b_res[12];
};

struct UvHit {
    short det, el, sign;
    float pos, drift, tdc, Y, eY, Z;
};

struct Stale {
    short det;
    float pos, drift;
};

// resolve_leftright_newhits walk over hits[0..n) with the scratch entry past
// the end given by `st` (H:714-780), then the singles (H:785-804).
__device__ __forceinline__ void walk_newhits(int n, UvHit *h, const Stale &st, float x0, float tx, float y0, float ty,
                                             float ex0, float etx, float ey0, float ety, const or_plane_t &P) {
    for (int i = 0; i < n;) {
        const int j = i + 1;
        const short di = h[i].det;
        const short dj = j < n ? h[j].det : st.det;
        if (abs(di - dj) != 1) {
            i += 1;
            continue;
        }
        const short sj = j < n ? h[j].sign : (short)0;
        if (h[i].sign * sj == 0) {
            const float pj = j < n ? h[j].pos : st.pos;
            const float drj = j < n ? h[j].drift : st.drift;
            const int k = lr_pair_newhits(x0, tx, y0, ty, ex0, etx, ey0, ety, di, dj, h[i].pos, h[i].drift, pj, drj, P,
                                          150.f);
            if (k >= 0) {
                h[i].sign = c_lrpossibility[k][0];
                if (j < n) h[j].sign = c_lrpossibility[k][1];
            }
        }
        i += 2;
    }
    for (int k = 0; k < n; ++k)
        if (!h[k].sign) h[k].sign = single_sign_newhits(x0, tx, y0, ty, h[k].det, h[k].pos, P);
}

// Index of the last station-3 hit when the walk pairs it with the first
// station-2 hit, else -1.  The walk's pairs depend only on plane ids.
__device__ __forceinline__ int cross_pair_index(int n3, const UvHit *h, int nuv) {
    for (int i = 0; i < n3;) {
        const int j = i + 1;
        if (j >= nuv) return -1;
        if (abs(h[i].det - h[j].det) != 1) {
            i += 1;
            continue;
        }
        if (j == n3) return i;
        i += 2;
    }
    return -1;
}

__global__ void __launch_bounds__(YZ_WARPS * 32)
    yz_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
              const uint8_t *__restrict__ toomany, int n_events, uint32_t *__restrict__ errw) {
    extern __shared__ __align__(16) unsigned char yz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(yz_smem);
    YzWarp *warps = reinterpret_cast<YzWarp *>(yz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    YzWarp &S = warps[w];

    for (long e = (long)blockIdx.x * YZ_WARPS + w; e < n_events; e += (long)gridDim.x * YZ_WARPS) {
        if (toomany[e]) continue;  // K:873-878
        const HitPlane p1y1 = hits_of(hv, e, DET_P1Y1), p1y2 = hits_of(hv, e, DET_P1Y2);
        const HitPlane p2y1 = hits_of(hv, e, DET_P2Y1), p2y2 = hits_of(hv, e, DET_P2Y2);
        HitPlane hod[3][2];
        for (int q = 0; q < 3; ++q)
            for (int c = 0; c < 2; ++c) hod[q][c] = hits_of(hv, e, c_hodoplanesx[q + 1][c]);

        for (int slot = 0; slot < OR_NSLOTS; ++slot) {
            const int ntr = min((int)tv.ntracks[e * OR_NSLOTS + slot], OR_SLOTCAP);
            if (ntr == 0) continue;
            const int st3 = 3 + (slot & 1);  // K:884
            // u2 u2' v2 v2' u3 u3' v3 v3' (K:910-984)
            const short dl[8] = {DET_U2, DET_UP2, DET_V2, DET_VP2, (short)det_u3(st3), (short)(det_u3(st3) - 1),
                                 (short)det_v3(st3), (short)(det_v3(st3) - 1)};
            HitPlane hc[8];
            for (int k = 0; k < 8; ++k) hc[k] = hits_of(hv, e, dl[k]);
            // scratch entries 4..7 as last written in this slot (sentinel start)
            Stale carry_st[4];
            for (int k = 0; k < 4; ++k) carry_st[k] = Stale{DET_SENTINEL, 0.f, 0.f};

            for (int it = 0; it < ntr; ++it) {
                float *T = trk_rec(tv, e, slot, it);
                const float x0 = T[OR_TRK_X0], tx = T[OR_TRK_TX], ex0 = T[OR_TRK_ERR_X0], etx = T[OR_TRK_ERR_TX];
                const int nhx = min((int)T[OR_TRK_NHITS], 4);  // XZ tracklets carry 2-4 hits
                // windowed pairs (K:1249-1283)
                int np[4];
                const int stid_of[4] = {2, 2, st3, st3}, proj_of[4] = {1, 2, 1, 2};
                bool overcap = false;
                for (int q = 0; q < 4; ++q) {
                    const int a = 2 * q;
                    const float za = P.z[dl[a]], zb = P.z[dl[a + 1]];
                    const float sp = P.spacing[dl[a]];
                    const float xmin = fminf((tx - etx) * za, (tx - etx) * zb) + x0 - ex0 - sp;
                    const float xmax = fmaxf((tx + etx) * za, (tx + etx) * zb) + x0 + ex0 + sp;
                    const float spacing = c_spacingplane[c_detsuperid[stid_of[q]][proj_of[q]]];
                    np[q] = window_pairs(hc[a], dl[a], hc[a + 1], dl[a + 1], spacing, xmin, xmax, P, S.pairs[q],
                                         YZ_PAIRCAP, S.W);
                    overcap |= np[q] > YZ_PAIRCAP;
                }
                if (lane == 0) T[OR_TRK_STID] = 3.f;  // K:1285
                const int nu2 = np[0], nv2 = np[1], nu3 = np[2], nv3 = np[3];
                if (overcap) {
                    if (lane == 0) atomicOr(errw, ERRW_CAPACITY);
                    continue;
                }
                if (nu2 == 0 || nu3 == 0 || nv2 == 0 || nv3 == 0) continue;
                // x hits of the tracklet (K:1300-1316)
                if (lane < nhx && lane < 4) {
                    const short d = (short)T[OR_TRK_HIT_DETID + lane];
                    const short ch = (short)T[OR_TRK_HIT_CHAN + lane];
                    S.xdd[lane] = T[OR_TRK_HIT_DRIFT + lane];
                    S.xhs[lane] = (short)T[OR_TRK_HIT_SIGN + lane];
                    S.xres[lane] = P.resolution[d];
                    S.xp1x[lane] = x_bep(d, ch, P);
                    S.xp1y[lane] = y_bep(d, ch, P);
                    S.xp1z[lane] = z_bep(d, ch, P);
                    S.xdpx[lane] = P.deltapx[d];
                    S.xdpy[lane] = P.deltapy[d];
                    S.xdpz[lane] = P.deltapz[d];
                }
                __syncwarp();
                const int C2 = nu2 * nv2;
                const long C = (long)nu3 * nv3 * C2;
                float run_min = 10000.1f;
                bool update = false;
                // sign-state carry of the current (u3,v3) iteration
                long cg = -1;
                bool cg_hasf = false, cg_hascross = false;
                short cg_sig[4] = {0, 0, 0, 0};
                short cg_cross = 0;

                for (long base = 0; base < C; base += 32) {
                    const long c = base + lane;
                    const bool valid = c < C;
                    const long g = valid ? c / C2 : -1 - (long)lane;
                    UvHit h[8];
                    int nuv = 0, n3 = 0;
                    bool v3ok = false, v2ok = false;
                    Stale own[4];
                    unsigned wmask = 0u;
                    float y0 = 0.f, ty = 0.f, ey0 = 0.f, ety = 0.f;
                    bool pass1 = false;
                    if (valid) {
                        const int iuv3 = (int)(c / C2), iuv2 = (int)(c - (long)iuv3 * C2);
                        const int iu3 = iuv3 % nu3, iv3 = iuv3 / nu3;
                        const int iu2 = iuv2 % nu2, iv2 = iuv2 / nu2;
                        const short2 pu3 = S.pairs[2][iu3], pv3 = S.pairs[3][iv3];
                        const short2 pu2 = S.pairs[0][iu2], pv2 = S.pairs[1][iv2];
                        // one load attempt (K:1326-1355); S2 attempts are recorded
                        // for the scratch-entry scan
                        auto attempt = [&](int lk, int hidx, bool record) {
                            UvHit &u = h[nuv];
                            u.det = dl[lk];
                            u.el = (short)hc[lk].chan(hidx);
                            u.tdc = hc[lk].tdc(hidx);
                            u.sign = 0;
                            u.drift = hc[lk].drift(hidx);
                            u.pos = hc[lk].pos(hidx);
                            u.Z = P.z[dl[lk]];
                            if (record && nuv >= 4 && nuv < 8) {
                                own[nuv - 4] = Stale{u.det, u.pos, u.drift};
                                wmask |= 1u << (nuv - 4);
                            }
                            float yy, ey;
                            if (calculate_y_uvhit(u.det, u.el, u.drift, 0, x0, tx, P, yy, ey)) {
                                u.Y = yy;
                                u.eY = ey;
                                ++nuv;
                            }
                        };
                        if (pu3.x >= 0) attempt(4, pu3.x, false);
                        if (pu3.y >= 0) attempt(5, pu3.y, false);
                        const int nhu3 = nuv;
                        if (nhu3 > 0) {
                            if (pv3.x >= 0) attempt(6, pv3.x, false);
                            if (pv3.y >= 0) attempt(7, pv3.y, false);
                            v3ok = nuv > nhu3;
                        }
                        n3 = nuv;
                        if (v3ok) {
                            if (pu2.x >= 0) attempt(0, pu2.x, true);
                            if (pu2.y >= 0) attempt(1, pu2.y, true);
                            if (nuv > n3) {
                                const int nb = nuv;
                                if (pv2.x >= 0) attempt(2, pv2.x, true);
                                if (pv2.y >= 0) attempt(3, pv2.y, true);
                                v2ok = nuv > nb;
                            }
                        }
                        if (v2ok) {  // K:1602-1611
                            Fit2 f;
                            for (int k = 0; k < nuv; ++k) f.add(h[k].Y, h[k].Z, h[k].eY);
                            f.solve(y0, ty, ey0, ety);
                            pass1 = !(fabsf(y0) > Y0_MAX + 2 * ey0 || fabsf(ty) > TY_MAX + 2 * ety);
                        }
                    }
                    // --- scratch entry past the hit count -----------------------
                    Stale st{DET_SENTINEL, 0.f, 0.f};
                    {
                        const int j = nuv;
                        const unsigned lt = lanemask_lt();
#pragma unroll
                        for (int k = 0; k < 4; ++k) {
                            const unsigned m = __ballot_sync(0xffffffffu, (wmask >> k) & 1u);
                            const int src = last_lane(m & lt);
                            const short sd = (short)__shfl_sync(0xffffffffu, (int)own[k].det, src < 0 ? 0 : src);
                            const float sp = __shfl_sync(0xffffffffu, own[k].pos, src < 0 ? 0 : src);
                            const float sdr = __shfl_sync(0xffffffffu, own[k].drift, src < 0 ? 0 : src);
                            if (j == k + 4) {
                                if ((wmask >> k) & 1u) st = own[k];
                                else if (src >= 0) st = Stale{sd, sp, sdr};
                                else st = carry_st[k];
                            }
                            const int lw = last_lane(m);
                            const short cd = (short)__shfl_sync(0xffffffffu, (int)own[k].det, lw < 0 ? 0 : lw);
                            const float cp = __shfl_sync(0xffffffffu, own[k].pos, lw < 0 ? 0 : lw);
                            const float cdr = __shfl_sync(0xffffffffu, own[k].drift, lw < 0 ? 0 : lw);
                            if (lw >= 0) carry_st[k] = Stale{cd, cp, cdr};
                        }
                    }
                    // --- station-3 sign state --------------------------------------
                    const unsigned seg = __match_any_sync(0xffffffffu, (unsigned long long)g);
                    const unsigned pm = __ballot_sync(0xffffffffu, pass1);
                    const bool carried_f = (g == cg) && cg_hasf;
                    const int fl = __ffs(pm & seg) - 1;
                    const bool is_first = pass1 && !carried_f && fl == lane;
                    // the first passing combination resolves from zero signs
                    if (is_first) walk_newhits(nuv, h, st, x0, tx, y0, ty, ex0, etx, ey0, ety, P);
                    // its station-3 signs, to every lane of the same iteration
                    short sig[4];
#pragma unroll
                    for (int k = 0; k < 4; ++k) {
                        const short mine = (k < n3) ? h[k].sign : (short)0;
                        const short v = (short)__shfl_sync(0xffffffffu, (int)mine, fl < 0 ? 0 : fl);
                        sig[k] = carried_f ? cg_sig[k] : v;
                    }
                    // cross pair (last station-3 hit, first station-2 hit)
                    int xi = -1;
                    short xval = 0;
                    bool xok = false;
                    if (pass1 && !is_first) {
                        xi = cross_pair_index(n3, h, nuv);
                        if (xi >= 0) {
                            const int k = lr_pair_newhits(x0, tx, y0, ty, ex0, etx, ey0, ety, h[xi].det,
                                                          h[xi + 1].det, h[xi].pos, h[xi].drift, h[xi + 1].pos,
                                                          h[xi + 1].drift, P, 150.f);
                            if (k >= 0) {
                                xok = true;
                                xval = c_lrpossibility[k][0];
                            }
                        }
                    }
                    const unsigned xm = __ballot_sync(0xffffffffu, xok);
                    const int xs = last_lane(xm & seg & lanemask_lt());
                    const short xprev = (short)__shfl_sync(0xffffffffu, (int)xval, xs < 0 ? 0 : xs);
                    bool pass = false;
                    float chi2 = 0.f;
                    float resid[12];
                    if (pass1 && !is_first) {
                        // station-3 signs at the start of this combination
                        for (int k = 0; k < n3 && k < 4; ++k) h[k].sign = sig[k];
                        if (n3 > 0) {
                            const int last3 = n3 - 1;
                            if (xs >= 0) h[last3].sign = xprev;
                            else if (g == cg && cg_hascross) h[last3].sign = cg_cross;
                        }
                        walk_newhits(nuv, h, st, x0, tx, y0, ty, ex0, etx, ey0, ety, P);
                    }
                    if (pass1) {
                        // refit gives the same y0/ty (same inputs); hard cut, K:1638
                        pass = !(fabsf(y0) > Y0_MAX || fabsf(ty) > TY_MAX);
                        if (pass) {
                            const int nprop = prop_hits(p1y1, P.z[DET_P1Y1], p1y2, P.z[DET_P1Y2], 5.08f, y0, ty) +
                                              prop_hits(p2y1, P.z[DET_P2Y1], p2y2, P.z[DET_P2Y2], 10.16f, y0, ty);
                            pass = nprop >= NPROP_MIN;
                        }
                        for (int q = 0; q < 3 && pass; ++q) {
                            pass = match_tracklet_to_hodo(q + 1, c_hodoplanesx[q + 1][0], hod[q][0], x0, y0, tx, ty,
                                                          ex0, ey0, etx, ety, P) ||
                                   match_tracklet_to_hodo(q + 1, c_hodoplanesx[q + 1][1], hod[q][1], x0, y0, tx, ty,
                                                          ex0, ey0, etx, ety, P);
                        }
                        if (pass) {  // chi2_track, H:1182-1204
                            for (int m = 0; m < nhx; ++m) {
                                resid[m] = residual_line(S.xp1x[m], S.xp1y[m], S.xp1z[m], S.xdpx[m], S.xdpy[m],
                                                         S.xdpz[m], S.xdd[m], S.xhs[m], x0, y0, tx, ty);
                                chi2 += resid[m] * resid[m] / S.xres[m] / S.xres[m];
                            }
                            for (int k = 0; k < nuv; ++k) {
                                const short d = h[k].det;
                                const float r = residual_line(x_bep(d, h[k].el, P), y_bep(d, h[k].el, P),
                                                              z_bep(d, h[k].el, P), P.deltapx[d], P.deltapy[d],
                                                              P.deltapz[d], h[k].drift, h[k].sign, x0, y0, tx, ty);
                                resid[nhx + k] = r;
                                chi2 += r * r / P.resolution[d] / P.resolution[d];
                            }
                        }
                    }
                    // --- carry of the sign state to the next chunk -----------------
                    {
                        const int last = last_lane(__ballot_sync(0xffffffffu, valid));
                        const long gl = __shfl_sync(0xffffffffu, g, last < 0 ? 0 : last);
                        const unsigned segl = __ballot_sync(0xffffffffu, valid && g == gl);
                        const int fnew = __ffs(__ballot_sync(0xffffffffu, is_first) & segl) - 1;
                        short ns[4];
#pragma unroll
                        for (int k = 0; k < 4; ++k) ns[k] = (short)__shfl_sync(0xffffffffu, (int)sig[k], fnew < 0 ? 0 : fnew);
                        const int xl = last_lane(xm & segl);
                        const short nx = (short)__shfl_sync(0xffffffffu, (int)xval, xl < 0 ? 0 : xl);
                        const bool cont = (gl == cg);
                        if (fnew >= 0) {
                            cg_hasf = true;
                            for (int k = 0; k < 4; ++k) cg_sig[k] = ns[k];
                        } else if (!cont) {
                            cg_hasf = false;
                        }
                        if (xl >= 0) {
                            cg_hascross = true;
                            cg_cross = nx;
                        } else if (!cont) {
                            cg_hascross = false;
                        }
                        cg = gl;
                    }
                    // --- best chi2, strict < in combination order (K:1778) ----------
                    const bool elig = pass && chi2 < run_min;
                    const unsigned key = elig ? __float_as_uint(chi2) : 0xffffffffu;
                    const unsigned kmin = __reduce_min_sync(0xffffffffu, key);
                    if (kmin != 0xffffffffu) {
                        const int win = __ffs(__ballot_sync(0xffffffffu, key == kmin)) - 1;
                        if (lane == win) {
                            S.b_nuv = nuv;
                            S.b_chi2 = chi2;
                            S.b_ty = ty;
                            S.b_y0 = y0;
                            S.b_ety = ety;
                            S.b_ey0 = ey0;
                            for (int n = 0; n < nuv; ++n) {
                                S.b_det[n] = h[n].det;
                                S.b_el[n] = h[n].el;
                                S.b_pos[n] = h[n].pos;
                                S.b_drift[n] = h[n].drift;
                                S.b_sign[n] = h[n].sign;
                                S.b_tdc[n] = h[n].tdc;
                            }
                            for (int n = 0; n < nhx + nuv; ++n) S.b_res[n] = resid[n];
                        }
                        run_min = __uint_as_float(kmin);
                        update = true;
                        __syncwarp();
                    }
                }
                if (update) {  // K:1804-1825
                    __syncwarp();
                    const int nuv = S.b_nuv;
                    if (lane == 0) {
                        T[OR_TRK_STID] = 5.f;
                        T[OR_TRK_NHITS] = (float)nhx + (float)nuv;
                        T[OR_TRK_CHI2] = S.b_chi2;
                        T[OR_TRK_TY] = S.b_ty;
                        T[OR_TRK_Y0] = S.b_y0;
                        T[OR_TRK_ERR_TY] = S.b_ety;
                        T[OR_TRK_ERR_Y0] = S.b_ey0;
                    }
                    if (lane < nuv) {
                        const int n = lane;
                        T[OR_TRK_HIT_DETID + nhx + n] = S.b_det[n];
                        T[OR_TRK_HIT_CHAN + nhx + n] = S.b_el[n];
                        T[OR_TRK_HIT_POS + nhx + n] = S.b_pos[n];
                        T[OR_TRK_HIT_DRIFT + nhx + n] = S.b_drift[n];
                        T[OR_TRK_HIT_SIGN + nhx + n] = S.b_sign[n];
                        T[OR_TRK_HIT_TDC + nhx + n] = S.b_tdc[n];
                        if (n < nhx) T[OR_TRK_HIT_RESID + n] = S.b_res[n];
                        T[OR_TRK_HIT_RESID + nhx + n] = S.b_res[nhx + n];
                    }
                }
                __syncwarp();
            }
        }
    }
}

size_t yz_smem_bytes() { return ((sizeof(or_plane_t) + 15) & ~size_t(15)) + sizeof(YzWarp) * YZ_WARPS; }

cudaError_t launch_yz(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, const uint8_t *toomany,
                      int n_events, uint32_t *errw, cudaStream_t stream, int sm_count) {
    if (n_events <= 0) return cudaSuccess;
    const size_t smem = yz_smem_bytes();
    cudaError_t err = cudaFuncSetAttribute(yz_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    long blocks = (n_events + YZ_WARPS - 1) / YZ_WARPS;
    const long cap = (long)sm_count * 8;
    if (blocks > cap) blocks = cap;
    yz_kernel<<<(unsigned)blocks, YZ_WARPS * 32, smem, stream>>>(d_plane, hv, tv, toomany, n_events, errw);
    return cudaGetLastError();
}

}  // namespace orgpu
