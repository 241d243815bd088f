// xz_kernel.cu -- station-2/3 XZ tracklets.
//
// Replaces gKernel_XZ_tracking<<<N,32>>> (OnlineReconstruction/
// reconstruction_kernels.cuh:182-855) with make_hitpairs_in_station_bins
// (reconstruction_helper.cuh:368-460) and the fit / left-right / prop / hodo
// helpers it calls.
//
// GPU layout: one warp per event.
//  1. X/X' hit pairs of station 2, 3+ and 3- are built with a lane grid over
//     (hit1, hit2); each bin's list keeps the reference order (pairs in
//     (i,j) order, then unpaired x, then unpaired x') through
//     __match_any_sync ranks.  A bin with more than 20 entries rejects the
//     event (K:359-375).
//  2. The reference splits the 28x28 bin space over 32 threads (K:217-219);
//     every thread enumerates 49 bin pairs and, in each, all (pair2, pair3)
//     candidates.  Here the candidates of all 32 thread groups are one
//     flattened index space (t, bin pair, candidate) evaluated 32 at a time.
//  3. The reference's per-thread scratch arrays persist across candidates,
//     and its left/right walk reads the entry just past the hit count when it
//     lands on the last hit (H:820-828).  That entry holds hit #2 (#3) of the
//     latest earlier candidate of the same thread with >= 3 (4) hits; a
//     segmented last-writer scan over the flattened candidates (ballot +
//     shuffle, carried across chunks) gives each lane exactly that data.
//  4. Surviving tracklets are compacted in order; the k-th tracklet of
//     station-3 half p goes to slot 2*(k%16)+p, position k/16 -- the
//     round-robin the reference's least-populated-slot balancing
//     (K:675-807) performs when adds come one at a time.
#include "or_device.cuh"

namespace orgpu {

constexpr int XZ_NCELLS = 32 * 49;
constexpr int XZ_MAXPLANEHITS = 200;

struct XzWarp {
    short2 pairs[3][28][MAXHITS_PROJ_X + 1];
    int np[3][28];
    uint8_t paired1[XZ_MAXPLANEHITS];
    uint8_t paired2[XZ_MAXPLANEHITS];
    int cell_prefix[XZ_NCELLS + 1];
};

// Append one (first, second) entry to bin `bin` of station q, in lane order.
__device__ __forceinline__ void xz_append(XzWarp &S, int q, bool take, int bin, int first, int second) {
    const unsigned act = __ballot_sync(0xffffffffu, take);
    if (!act) return;
    const int key = take ? bin : -1 - (int)lane_id();  // non-takers form singleton groups
    const unsigned peers = __match_any_sync(0xffffffffu, key);
    int base = 0;
    if (take) {
        base = S.np[q][bin];
        const int slot = base + __popc(peers & lanemask_lt());
        if (slot <= MAXHITS_PROJ_X) S.pairs[q][bin][slot] = make_short2((short)first, (short)second);
    }
    __syncwarp();
    if (take && (peers & lanemask_lt()) == 0u) S.np[q][bin] = base + __popc(peers);
    __syncwarp();
}

// make_hitpairs_in_station_bins over all 28 bins of one station
static __device__ void xz_pairs(XzWarp &S, int q, int st, const HitPlane &h1, const HitPlane &h2) {
    const int lane = lane_id();
    const int n1 = min(h1.n, XZ_MAXPLANEHITS), n2 = min(h2.n, XZ_MAXPLANEHITS);
    for (int b = lane; b < 28; b += 32) S.np[q][b] = 0;
    for (int i = lane; i < n1; i += 32) S.paired1[i] = 0;
    for (int j = lane; j < n2; j += 32) S.paired2[j] = 0;
    __syncwarp();
    const float spacing = c_spacingplane[c_detsuperid[st][0]];
    const int nn = n1 * n2;
    for (int base = 0; base < nn; base += 32) {
        const int c = base + lane;
        bool take = false;
        int bin = -1, i = 0, j = 0;
        if (c < nn) {
            i = c / n2;
            j = c - i * n2;
            if (!(fabsf(h1.pos(i) - h2.pos(j)) > spacing)) {
                S.paired1[i] = 1;
                S.paired2[j] = 1;
                bin = x_bin_of(st, h1.chan(i));
                take = bin >= 0;
            }
        }
        xz_append(S, q, take, bin, i, j);
    }
    __syncwarp();
    for (int base = 0; base < n1; base += 32) {
        const int i = base + lane;
        int bin = -1;
        bool take = false;
        if (i < n1 && !S.paired1[i]) {
            bin = x_bin_of(st, h1.chan(i));
            take = bin >= 0;
        }
        xz_append(S, q, take, bin, i, -1);
    }
    for (int base = 0; base < n2; base += 32) {
        const int j = base + lane;
        int bin = -1;
        bool take = false;
        if (j < n2 && !S.paired2[j]) {
            bin = x_bin_of(st, h2.chan(j));
            take = bin >= 0;
        }
        xz_append(S, q, take, bin, -1, j);
    }
}

struct XHit {
    short det;
    short el;
    float X, Z, drift, tdc, w;
};

template <int W>
__global__ void __launch_bounds__(W * 32)
    xz_kernel(const or_plane_t *__restrict__ gplane, or_hits_view_t hv, or_tracks_view_t tv,
              int32_t *__restrict__ ntracklets, uint8_t *__restrict__ toomany, int n_events) {
    extern __shared__ __align__(16) unsigned char xz_smem[];
    or_plane_t &P = *reinterpret_cast<or_plane_t *>(xz_smem);
    XzWarp *warps = reinterpret_cast<XzWarp *>(xz_smem + ((sizeof(or_plane_t) + 15) & ~size_t(15)));
    load_plane_smem(&P, gplane);
    __syncthreads();
    const int w = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    XzWarp &S = warps[w];

    for (long e = (long)blockIdx.x * W + w; e < n_events; e += (long)gridDim.x * W) {
        uint16_t *nt = tv.ntracks + e * OR_NSLOTS;
        if (toomany[e]) {  // K:195-200
            nt[lane] = 0;
            continue;
        }
        // --- 1. pairs -------------------------------------------------------
        HitPlane hx[3], hxp[3];
        const int detx[3] = {DET_X2, det_x3(3), det_x3(4)};
        for (int q = 0; q < 3; ++q) {
            hx[q] = hits_of(hv, e, detx[q]);
            hxp[q] = hits_of(hv, e, detx[q] - 1);
            xz_pairs(S, q, 2 + q, hx[q], hxp[q]);
        }
        __syncwarp();
        bool over = false;
        for (int q = 0; q < 3; ++q)
            if (lane < 28 && S.np[q][lane] > MAXHITS_PROJ_X) over = true;
        over = __any_sync(0xffffffffu, over) || hx[0].n > XZ_MAXPLANEHITS || hxp[0].n > XZ_MAXPLANEHITS ||
               hx[1].n > XZ_MAXPLANEHITS || hxp[1].n > XZ_MAXPLANEHITS || hx[2].n > XZ_MAXPLANEHITS ||
               hxp[2].n > XZ_MAXPLANEHITS;
        if (over) {
            nt[lane] = 0;
            if (lane == 0) {
                toomany[e] = 1;
                ntracklets[e] = 0;
            }
            continue;
        }
        // --- 2. candidate index space ---------------------------------------
        int carry = 0;
        for (int base = 0; base < XZ_NCELLS; base += 32) {
            const int cell = base + lane;
            int cnt = 0;
            if (cell < XZ_NCELLS) {
                const int t = cell / 49, i = cell - t * 49;
                const int b2 = i % 7, b3 = i / 7;
                cnt = S.np[0][(t / 8) * 7 + b2] * S.np[1 + (t & 1)][((t % 8) / 2) * 7 + b3];
            }
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int v = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += v;
            }
            if (cell < XZ_NCELLS) S.cell_prefix[cell] = carry + incl - cnt;
            carry += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) S.cell_prefix[XZ_NCELLS] = carry;
        __syncwarp();
        const int total = carry;

        // planes for the gates
        const HitPlane p1x1 = hits_of(hv, e, DET_P1X1), p1x2 = hits_of(hv, e, DET_P1X2);
        const HitPlane p2x1 = hits_of(hv, e, DET_P2X1), p2x2 = hits_of(hv, e, DET_P2X2);
        HitPlane hod[3][2];
        for (int q = 0; q < 3; ++q)
            for (int c = 0; c < 2; ++c) hod[q][c] = hits_of(hv, e, c_hodoplanesx[q + 1][c]);

        // stale scratch state carried across chunks (last writer of entries 2, 3)
        int carry_t = -1;
        short cdet2 = DET_SENTINEL, cdet3 = DET_SENTINEL;
        float cX2 = 0.f, cdr2 = 0.f, cX3 = 0.f, cdr3 = 0.f;
        int kpar0 = 0, kpar1 = 0;

        // --- 3. candidates --------------------------------------------------
        for (int base = 0; base < total; base += 32) {
            const int c = base + lane;
            const bool valid = c < total;
            int t = 32 + lane;  // distinct keys for invalid lanes
            int nh = 0;
            XHit hit[4];
            int cell = 0;
            if (valid) {
                int lo = 0, hi = XZ_NCELLS - 1;  // largest cell with prefix <= c
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (S.cell_prefix[mid] <= c) lo = mid; else hi = mid - 1;
                }
                cell = lo;
                t = cell / 49;
                const int i = cell - t * 49;
                const int b2 = i % 7, b3 = i / 7;
                const int bin2 = (t / 8) * 7 + b2, bin3 = ((t % 8) / 2) * 7 + b3;
                const int q3 = 1 + (t & 1);
                const int nx2 = S.np[0][bin2];
                const int ix = c - S.cell_prefix[cell];
                const int ix2 = ix % nx2, ix3 = ix / nx2;
                const short2 p2 = S.pairs[0][bin2][ix2], p3 = S.pairs[q3][bin3][ix3];
                const int dets[4] = {DET_X2, DET_XP2, det_x3(2 + q3), det_x3(2 + q3) - 1};
                const int idx[4] = {p2.x, p2.y, p3.x, p3.y};
                const HitPlane *hp[4] = {&hx[0], &hxp[0], &hx[q3], &hxp[q3]};
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    if (idx[k] < 0) continue;
                    XHit &h = hit[nh];
                    h.det = (short)dets[k];
                    h.el = (short)hp[k]->chan(idx[k]);
                    h.tdc = hp[k]->tdc(idx[k]);
                    h.drift = hp[k]->drift(idx[k]);
                    h.w = P.resolution[dets[k]];
                    calculate_xz_fy(h.det, h.el, h.drift, 0, 0.f, 0.f, P, h.X, h.Z);
                    ++nh;
                }
            }
            // segmented last-writer scan of scratch entries 2 and 3
            const unsigned same_t = __match_any_sync(0xffffffffu, t);
            const unsigned w2 = __ballot_sync(0xffffffffu, valid && nh >= 3);
            const unsigned w3 = __ballot_sync(0xffffffffu, valid && nh == 4);
            const short my_d2 = nh >= 3 ? hit[2].det : DET_SENTINEL;
            const float my_X2 = nh >= 3 ? hit[2].X : 0.f, my_dr2 = nh >= 3 ? hit[2].drift : 0.f;
            const short my_d3 = nh == 4 ? hit[3].det : DET_SENTINEL;
            const float my_X3 = nh == 4 ? hit[3].X : 0.f, my_dr3 = nh == 4 ? hit[3].drift : 0.f;
            const int l2 = last_lane(w2 & same_t & lanemask_lt());
            const int l3 = last_lane(w3 & same_t & lanemask_lt());
            const short sd2 = (short)__shfl_sync(0xffffffffu, (int)my_d2, l2 < 0 ? 0 : l2);
            const float sX2 = __shfl_sync(0xffffffffu, my_X2, l2 < 0 ? 0 : l2);
            const float sdr2 = __shfl_sync(0xffffffffu, my_dr2, l2 < 0 ? 0 : l2);
            const short sd3 = (short)__shfl_sync(0xffffffffu, (int)my_d3, l3 < 0 ? 0 : l3);
            const float sX3 = __shfl_sync(0xffffffffu, my_X3, l3 < 0 ? 0 : l3);
            const float sdr3 = __shfl_sync(0xffffffffu, my_dr3, l3 < 0 ? 0 : l3);
            short st_d2, st_d3;
            float st_X2, st_dr2, st_X3, st_dr3;
            if (l2 >= 0) {
                st_d2 = sd2; st_X2 = sX2; st_dr2 = sdr2;
            } else if (t == carry_t) {
                st_d2 = cdet2; st_X2 = cX2; st_dr2 = cdr2;
            } else {
                st_d2 = DET_SENTINEL; st_X2 = 0.f; st_dr2 = 0.f;
            }
            if (l3 >= 0) {
                st_d3 = sd3; st_X3 = sX3; st_dr3 = sdr3;
            } else if (t == carry_t) {
                st_d3 = cdet3; st_X3 = cX3; st_dr3 = cdr3;
            } else {
                st_d3 = DET_SENTINEL; st_X3 = 0.f; st_dr3 = 0.f;
            }
            // carry for the next chunk: state after the last valid lane
            {
                const int last = last_lane(__ballot_sync(0xffffffffu, valid));
                const int tl = __shfl_sync(0xffffffffu, t, last);
                const unsigned seg = __ballot_sync(0xffffffffu, valid && t == tl);
                const int a2 = last_lane(w2 & seg), a3 = last_lane(w3 & seg);
                const short nd2 = (short)__shfl_sync(0xffffffffu, (int)my_d2, a2 < 0 ? 0 : a2);
                const float nX2 = __shfl_sync(0xffffffffu, my_X2, a2 < 0 ? 0 : a2);
                const float ndr2 = __shfl_sync(0xffffffffu, my_dr2, a2 < 0 ? 0 : a2);
                const short nd3 = (short)__shfl_sync(0xffffffffu, (int)my_d3, a3 < 0 ? 0 : a3);
                const float nX3 = __shfl_sync(0xffffffffu, my_X3, a3 < 0 ? 0 : a3);
                const float ndr3 = __shfl_sync(0xffffffffu, my_dr3, a3 < 0 ? 0 : a3);
                const bool cont = (tl == carry_t);
                if (a2 >= 0) { cdet2 = nd2; cX2 = nX2; cdr2 = ndr2; }
                else if (!cont) { cdet2 = DET_SENTINEL; cX2 = 0.f; cdr2 = 0.f; }
                if (a3 >= 0) { cdet3 = nd3; cX3 = nX3; cdr3 = ndr3; }
                else if (!cont) { cdet3 = DET_SENTINEL; cX3 = 0.f; cdr3 = 0.f; }
                carry_t = tl;
            }

            // --- per-candidate gates (K:547-672) -------------------------------
            bool pass = false;
            float x0 = 0.f, tx = 0.f, ex0 = 0.f, etx = 0.f;
            short sign[4] = {0, 0, 0, 0};
            if (valid) {
                Fit2 f;
                for (int k = 0; k < nh; ++k) f.add(hit[k].X, hit[k].Z, hit[k].w);
                f.solve(x0, tx, ex0, etx);
                pass = !(fabsf(x0) > X0_MAX + 2 * ex0 || fabsf(tx) > TX_MAX + 2 * etx);
                if (pass) {
                    // resolve_leftright_xhits walk (H:820-871)
                    for (int n = 0; n < nh;) {
                        const int j = n + 1;
                        const short di = hit[n].det;
                        short dj;
                        float Xj, drj;
                        if (j < nh) {
                            dj = hit[j].det; Xj = hit[j].X; drj = hit[j].drift;
                        } else if (j == 2) {
                            dj = st_d2; Xj = st_X2; drj = st_dr2;
                        } else if (j == 3) {
                            dj = st_d3; Xj = st_X3; drj = st_dr3;
                        } else {
                            dj = DET_SENTINEL; Xj = 0.f; drj = 0.f;
                        }
                        if (abs(di - dj) != 1) {
                            n += 1;
                            continue;
                        }
                        const int k = lr_pair_xhits(x0, tx, ex0, etx, di, dj, hit[n].X, hit[n].drift, Xj, drj, P.z,
                                                    150.f);
                        if (k >= 0) {
                            sign[n] = c_lrpossibility[k][0];
                            if (j < nh) sign[j] = c_lrpossibility[k][1];
                        }
                        n += 2;
                    }
                    for (int k = 0; k < nh; ++k)
                        if (!sign[k]) sign[k] = single_sign_xhits(x0, tx, hit[k].det, hit[k].X, P.z);
                    Fit2 g;
                    for (int k = 0; k < nh; ++k) g.add_drift(hit[k].X, hit[k].drift, sign[k], hit[k].Z, hit[k].w);
                    g.solve(x0, tx, ex0, etx);
                    pass = !(fabsf(x0) > X0_MAX || fabsf(tx) > TX_MAX);
                }
                if (pass) {
                    const int nprop = prop_hits(p1x1, P.z[DET_P1X1], p1x2, P.z[DET_P1X2], 5.08f, x0, tx) +
                                      prop_hits(p2x1, P.z[DET_P2X1], p2x2, P.z[DET_P2X2], 7.62f, x0, tx);
                    pass = nprop >= NPROP_MIN;
                }
                for (int q = 0; q < 3 && pass; ++q) {
                    pass = match_track_XZ_to_hodo(q + 1, c_hodoplanesx[q + 1][0], hod[q][0], x0, tx, ex0, etx, P.z) ||
                           match_track_XZ_to_hodo(q + 1, c_hodoplanesx[q + 1][1], hod[q][1], x0, tx, ex0, etx, P.z);
                }
            }
            // --- 4. ordered output ------------------------------------------
            const unsigned m0 = __ballot_sync(0xffffffffu, pass && (t & 1) == 0);
            const unsigned m1 = __ballot_sync(0xffffffffu, pass && (t & 1) == 1);
            if (pass) {
                const int par = t & 1;
                const int k = (par ? kpar1 : kpar0) + __popc((par ? m1 : m0) & lanemask_lt());
                const int slot = 2 * (k % 16) + par, posn = k / 16;
                if (posn < OR_SLOTCAP) {
                    float *r = trk_rec(tv, e, slot, posn);
                    const int i = cell - t * 49;
                    for (int f = 0; f < OR_NTRKPARAM; ++f) r[f] = 0.f;
                    r[OR_TRK_STID] = (float)(t + 32 * i);
                    r[OR_TRK_THREAD] = (float)t;
                    r[OR_TRK_NHITS] = (float)nh;
                    r[OR_TRK_TX] = tx;
                    r[OR_TRK_X0] = x0;
                    r[OR_TRK_ERR_TX] = etx;
                    r[OR_TRK_ERR_X0] = ex0;
                    for (int n = 0; n < nh; ++n) {
                        r[OR_TRK_HIT_DETID + n] = (float)hit[n].det;
                        r[OR_TRK_HIT_CHAN + n] = (float)hit[n].el;
                        r[OR_TRK_HIT_POS + n] = hit[n].X;
                        r[OR_TRK_HIT_DRIFT + n] = hit[n].drift;
                        r[OR_TRK_HIT_SIGN + n] = (float)sign[n];
                        r[OR_TRK_HIT_TDC + n] = hit[n].tdc;
                    }
                }
            }
            kpar0 += __popc(m0);
            kpar1 += __popc(m1);
        }
        // --- 5. counts and overflow (K:812-839) -----------------------------
        const int ntot = kpar0 + kpar1;
        const bool full = ntot >= OR_TRKMAX || kpar0 > 16 * OR_SLOTCAP || kpar1 > 16 * OR_SLOTCAP;
        {
            const int par = lane & 1, m = lane >> 1;
            const int K = par ? kpar1 : kpar0;
            nt[lane] = full ? 0 : (uint16_t)(K > m ? (K - m + 15) / 16 : 0);
        }
        if (lane == 0) {
            ntracklets[e] = ntot;
            if (full) toomany[e] = 1;
        }
    }
}

size_t xz_smem_bytes(int warps) {
    return ((sizeof(or_plane_t) + 15) & ~size_t(15)) + sizeof(XzWarp) * (size_t)warps;
}

template <int W>
static cudaError_t xz_launch(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, int32_t *ntracklets,
                             uint8_t *toomany, int n_events, cudaStream_t stream, int sm_count) {
    const size_t smem = xz_smem_bytes(W);
    cudaError_t err = smem_attr_once((const void *)xz_kernel<W>, (int)smem);
    if (err != cudaSuccess) return err;
    long blocks = (n_events + W - 1) / W;
    const long cap = (long)sm_count * (32 / W > 0 ? 32 / W : 1);
    if (blocks > cap) blocks = cap;
    xz_kernel<W><<<(unsigned)blocks, W * 32, smem, stream>>>(d_plane, hv, tv, ntracklets, toomany, n_events);
    return cudaGetLastError();
}

// `warps` = events per CTA: 1, 2, 4 or 8 (the per-warp scratch is too large for 16)
cudaError_t launch_xz(const or_plane_t *d_plane, or_hits_view_t hv, or_tracks_view_t tv, int32_t *ntracklets,
                      uint8_t *toomany, int n_events, cudaStream_t stream, int sm_count, int warps) {
    if (n_events <= 0) return cudaSuccess;
    switch (warps) {
    case 1: return xz_launch<1>(d_plane, hv, tv, ntracklets, toomany, n_events, stream, sm_count);
    case 2: return xz_launch<2>(d_plane, hv, tv, ntracklets, toomany, n_events, stream, sm_count);
    case 8: return xz_launch<8>(d_plane, hv, tv, ntracklets, toomany, n_events, stream, sm_count);
    default: return xz_launch<4>(d_plane, hv, tv, ntracklets, toomany, n_events, stream, sm_count);
    }
}

}  // namespace orgpu
