// Discrete adjoint of one FMM force evaluation (vector-Jacobian product),
// with the tree and every interaction list frozen at the forward evaluation.
//
// For S = sum_i mu_i . a_i with a_i = G q_i/m_i E_i the product is taken
// operator by operator, in reverse:
//   near field  gx_k += sum_l T(r_kl) (q_k nu_l - q_l nu_k),  gq_k += nu_l . K(x_k - x_l)
//               (nu_i = G q_i/m_i mu_i, K(r) = r/s^3/2, T = dK/dr); the near-field pair set
//               is symmetric, so both the target and the source role of particle k are
//               gathered in k's own list: no scatter, no atomics;
//   L2P         gx_k += H(L) nu_k (Hessian of the local expansion) and
//               lamL(leaf) = sum_k sum_d nu_k,d y^(n-e_d)/(n-e_d)!;
//   L2L^T       an M2M pass on lamL (children -> parent, same shift operator);
//   M2L^T       the forward M2L kernel run on lamL over the same (symmetric) far-field
//               lists gives lamM (the operator's transpose has the forward form);
//   M2M^T       an L2L pass on lamM (parent -> children);
//   P2M^T       gq_k += psi_lamM(y_k), gx_k += q_k grad psi_lamM(y_k) (an L2P of lamM);
//   prefactor   gq_k += mu_k . a_k / q_k, gm_k -= mu_k . a_k / m_k.
// Cell centres are geometric, so M2M, M2L and L2L are constant linear maps.
#pragma once

namespace nbfmm {

struct AdjArgs {
    int64_t n;
    const uint32_t* ids;              // sorted row -> input index
    const void *lv, *q, *m, *ax, *ay, *az;   // R*: lv (input order, 3n), q/m/a (sorted)
    double c, G;                      // mu = c * lv
    void* nu;                         // S4* (sorted)
    void *gx, *gq, *gm;               // R* accumulators (input order; gx 3n)
};

template <int MODE>
__global__ void __launch_bounds__(256) k_adj_prep(AdjArgs A) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S4 S4;
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i >= A.n) return;
    const uint32_t id = A.ids[i];
    const R* lv = (const R*)A.lv;
    const R c = (R)A.c;
    const R mx = c * lv[3 * id], my = c * lv[3 * id + 1], mz = c * lv[3 * id + 2];
    const R qi = ((const R*)A.q)[i], mi = ((const R*)A.m)[i];
    const R f = (R)A.G * qi / mi;
    S4 v;
    v.x = (decltype(v.x))(f * mx); v.y = (decltype(v.y))(f * my); v.z = (decltype(v.z))(f * mz); v.w = 0;
    ((S4*)A.nu)[i] = v;
    const R mua = mx * ((const R*)A.ax)[i] + my * ((const R*)A.ay)[i] + mz * ((const R*)A.az)[i];
    if (qi != R(0)) ((R*)A.gq)[id] += mua / qi;
    ((R*)A.gm)[id] -= mua / mi;
}

// transpose of L2P: lamL_n of each leaf (lane per coefficient, like k_p2m)
template <int MODE, int P>
__global__ void __launch_bounds__(128) k_adj_l2pT(int64_t nleaves, const uint32_t* __restrict__ leaves,
                                                  const NodeRec* __restrict__ nodes,
                                                  const typename Prec<MODE>::S4* __restrict__ src,
                                                  const typename Prec<MODE>::S4* __restrict__ nu,
                                                  typename Prec<MODE>::H* __restrict__ lamL) {
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    constexpr int NPL = (T + 31) / 32;
    __shared__ S pw[4][32][3][P + 1];
    __shared__ S sn[4][32][3];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t w = (int64_t)blockIdx.x * 4 + wib;
    if (w >= nleaves) return;
    const uint32_t k = leaves[w];
    const NodeRec nd = nodes[k];
    int ex[NPL][3];
    S acc[NPL];
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        acc[j] = S(0);
        const int a = lane + 32 * j, aa = a < T ? a : 0;
        ex[j][0] = nb_mi[aa][0]; ex[j][1] = nb_mi[aa][1]; ex[j][2] = nb_mi[aa][2];
    }
    const uint32_t end = nd.begin + nd.count;
    for (uint32_t base = nd.begin; base < end; base += 32) {
        const uint32_t i = base + lane;
        if (i < end) {
            const typename Prec<MODE>::S4 y = src[i], v = nu[i];
            const S yy[3] = {y.x, y.y, y.z};
#pragma unroll
            for (int d = 0; d < 3; ++d) {
                S p = S(1);
#pragma unroll
                for (int e = 0; e <= P; ++e) { pw[wib][lane][d][e] = p; p *= yy[d]; }
            }
            sn[wib][lane][0] = v.x; sn[wib][lane][1] = v.y; sn[wib][lane][2] = v.z;
        }
        __syncwarp();
        const int cnt = end - base < 32 ? (int)(end - base) : 32;
        for (int jj = 0; jj < cnt; ++jj) {
#pragma unroll
            for (int j = 0; j < NPL; ++j) {
                const int nx = ex[j][0], ny = ex[j][1], nz = ex[j][2];
                S t = S(0);
                if (nx) t = nb_fma(sn[wib][jj][0] * (S)nx, pw[wib][jj][0][nx - 1] * pw[wib][jj][1][ny] * pw[wib][jj][2][nz], t);
                if (ny) t = nb_fma(sn[wib][jj][1] * (S)ny, pw[wib][jj][0][nx] * pw[wib][jj][1][ny - 1] * pw[wib][jj][2][nz], t);
                if (nz) t = nb_fma(sn[wib][jj][2] * (S)nz, pw[wib][jj][0][nx] * pw[wib][jj][1][ny] * pw[wib][jj][2][nz - 1], t);
                acc[j] += t;
            }
        }
        __syncwarp();
    }
#pragma unroll
    for (int j = 0; j < NPL; ++j) {
        const int a = lane + 32 * j;
        if (a < T) {
            const H v = (H)acc[j] * (H)nb_invfact[a];
            lamL[(int64_t)k * TM + a] = v;
        }
    }
}

struct AdjP2PArgs {
    const uint32_t* leaves;
    int64_t nleaves;
    int64_t nnodes, n;        // node and particle counts (index checks of the debug build)
    const NodeRec* nodes;
    const BoxDev* box;
    const void* src;          // S4* (offset from the leaf centre, q)
    const void* nu;           // S4*
    const void* L;            // H*: forward local expansions (stride T)
    const void* lamM;         // H*: adjoint multipoles (stride T)
    const uint32_t *p2p_off, *p2p_cnt, *p2p_list;
    const uint32_t* work_off;
    int64_t nwork;
    const uint32_t* part_off;
    void* part;               // R[4] per (chunk, target) of multi-chunk leaves
    void* near;               // R[4] per particle (sorted) of single-chunk leaves
    const uint32_t* ids;
    void *gx, *gq;            // R* accumulators (input order)
    double eps2;
};

// far-field part of the adjoint at one particle + accumulation into the input-order sums
template <int MODE, int P>
__device__ __forceinline__ void adj_epilogue(const AdjP2PArgs& A, uint32_t i, const typename Prec<MODE>::S* sL,
                                             const typename Prec<MODE>::S* sM, typename Prec<MODE>::S4 yi,
                                             typename Prec<MODE>::S4 ni, typename Prec<MODE>::R gx,
                                             typename Prec<MODE>::R gy, typename Prec<MODE>::R gz,
                                             typename Prec<MODE>::R gq) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    S hx, hy, hz;
    Ops<S, P>::l2p_hess(sL, yi.x, yi.y, yi.z, ni.x, ni.y, ni.z, hx, hy, hz);
    S fx, fy, fz, fp;
    Ops<S, P>::l2p(sM, yi.x, yi.y, yi.z, fx, fy, fz, fp);
    const uint32_t id = A.ids[i];
    R* GX = (R*)A.gx;
    R* GQ = (R*)A.gq;
    const R qi = (R)yi.w;
    GX[3 * id] += gx + (R)hx + qi * (R)fx;
    GX[3 * id + 1] += gy + (R)hy + qi * (R)fy;
    GX[3 * id + 2] += gz + (R)hz + qi * (R)fz;
    GQ[id] += gq + (R)fp;
}

constexpr int ADJ_WARPS = 4;

// lanes per target group and targets per lane of the adjoint near field, per leaf-size class
template <int CLS> struct AdjShape;
template <> struct AdjShape<0> { static constexpr int CT = 4, TPL = 2; };
template <> struct AdjShape<1> { static constexpr int CT = 8, TPL = 2; };
template <> struct AdjShape<2> { static constexpr int CT = 8, TPL = 3; };
template <> struct AdjShape<3> { static constexpr int CT = 16, TPL = 2; };
template <> struct AdjShape<4> { static constexpr int CT = 16, TPL = 3; };
template <> struct AdjShape<5> { static constexpr int CT = 32, TPL = 2; };

// One warp's share of an adjoint near-field work item: every target of the leaf (TPL per lane, CT
// lanes per group) against the partner leaves [s_lo, s_hi) of its list.  Per target k the pair
// sums are kept as
//   U = sum nu_l / s^3/2,  V = sum q_l / s^3/2,  W = sum r (r . w) / s^5/2,
//   gq = -sum (nu_l . r) / s^3/2   (r = x_l - x_k, w = q_k nu_l - q_l nu_k)
// and gx_k = q_k U - V nu_k - 3 W; the self pair is skipped.  Results go to the per-particle
// buffer (single-chunk leaves) or the chunk partials; k_adj_finish adds the far-field terms.
template <int MODE, bool GUARD, int CT, int TPL>
__device__ __forceinline__ void adj_item(const AdjP2PArgs& A, typename Prec<MODE>::S4* tx,
                                         typename Prec<MODE>::S4* tn, uint32_t k, const NodeRec& nt, int64_t li,
                                         uint32_t chunk, uint32_t nchunk, uint32_t s_lo, uint32_t s_hi) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::S4 S4;
    constexpr bool KH = Prec<MODE>::kahan;
    constexpr int NG = 32 / CT;
    constexpr int TILE = P2P_WTILE / NG < 32 ? P2P_WTILE / NG : 32;
    static_assert(NG * (TILE + 1) <= P2P_WROWS, "group tiles exceed the warp's shared rows");
    const int lane = lane_id();
    const int grp = lane / CT, gl = lane % CT;
    S4* gx_t = tx + grp * (TILE + 1);
    S4* gn_t = tn + grp * (TILE + 1);
    const double unit = A.box->unit;
    const S4* src = (const S4*)A.src;
    const S4* nu = (const S4*)A.nu;
    const uint32_t cnt_t = nt.count;
    const uint32_t loff = A.p2p_off[k];
    const S eps2 = (S)A.eps2;
    S4 zero4;
    zero4.x = 0; zero4.y = 0; zero4.z = 0; zero4.w = 0;
    for (uint32_t tc = 0; tc < cnt_t; tc += TPL * CT) {
        uint32_t ti[TPL], ii[TPL];
        bool tv[TPL];
        S4 y[TPL], nk[TPL];
        S sum[TPL][8], cmp[TPL][8];
#pragma unroll
        for (int j = 0; j < TPL; ++j) {
            ti[j] = tc + gl + j * CT;
            tv[j] = ti[j] < cnt_t;
            ii[j] = nt.begin + (tv[j] ? ti[j] : 0);
            y[j] = src[ii[j]];
            nk[j] = nu[ii[j]];
#pragma unroll
            for (int q = 0; q < 8; ++q) { sum[j][q] = 0; cmp[j][q] = 0; }
        }
        for (uint32_t base = s_lo; base < s_hi; base += 32) {
            const uint32_t nbat = min(32u, s_hi - base);
            uint32_t my_s = 0, my_beg = 0, my_cnt = 0;
            S my_dx = 0, my_dy = 0, my_dz = 0;
            if ((uint32_t)lane < nbat) {
                my_s = NB_IDX(A.p2p_list[loff + base + lane], A.nnodes, NB_SITE_ADJ);
                const NodeRec sn = A.nodes[my_s];
                my_beg = NB_IDX(sn.begin, A.n, NB_SITE_ADJ);
                my_cnt = NB_IDX(sn.count, A.n + 1 - my_beg, NB_SITE_ADJ);
                disp_s<S>(sn, nt, unit, my_dx, my_dy, my_dz);
            }
            // partners of this batch in descending particle count (as in the forward near field)
            {
                const uint32_t key = (min(my_cnt, 1u << 26) << 5) | (31u - (uint32_t)lane);
                const int from = 31 - (int)(warp_sort_desc(key) & 31u);
                my_s = __shfl_sync(0xffffffffu, my_s, from);
                my_beg = __shfl_sync(0xffffffffu, my_beg, from);
                my_cnt = __shfl_sync(0xffffffffu, my_cnt, from);
                my_dx = __shfl_sync(0xffffffffu, my_dx, from);
                my_dy = __shfl_sync(0xffffffffu, my_dy, from);
                my_dz = __shfl_sync(0xffffffffu, my_dz, from);
            }
            const uint32_t rounds = (nbat + NG - 1) / NG;
            for (uint32_t rr = 0; rr < rounds; ++rr) {
                const uint32_t q = rr * NG + grp;
                const uint32_t qs = q & 31;
                const uint32_t s_id = __shfl_sync(0xffffffffu, my_s, qs);
                const uint32_t beg = __shfl_sync(0xffffffffu, my_beg, qs);
                const uint32_t scnt0 = __shfl_sync(0xffffffffu, my_cnt, qs);
                const S dx = __shfl_sync(0xffffffffu, my_dx, qs), dy = __shfl_sync(0xffffffffu, my_dy, qs),
                        dz = __shfl_sync(0xffffffffu, my_dz, qs);
                const uint32_t scnt = q < nbat ? scnt0 : 0u;
                // the round's largest partner: partners are sorted by particle count, so it is the first
                const uint32_t mx = __shfl_sync(0xffffffffu, my_cnt, (rr * NG) & 31);
                const bool self = s_id == k && q < nbat;
                S xs[TPL][3];
#pragma unroll
                for (int j = 0; j < TPL; ++j) { xs[j][0] = y[j].x - dx; xs[j][1] = y[j].y - dy; xs[j][2] = y[j].z - dz; }
                for (uint32_t t0 = 0; t0 < mx; t0 += TILE) {
                    for (int e = gl; e < TILE; e += CT) {
                        const uint32_t jj = t0 + e;
                        gx_t[e] = jj < scnt ? src[beg + jj] : zero4;
                        gn_t[e] = jj < scnt ? nu[beg + jj] : zero4;
                    }
                    __syncwarp();
                    const int nj = scnt > t0 ? min((int)(scnt - t0), TILE) : 0;
                    int selfe[TPL];
#pragma unroll
                    for (int j = 0; j < TPL; ++j) selfe[j] = self ? (int)ti[j] - (int)t0 : -1;
                    S p[TPL][8];
#pragma unroll
                    for (int j = 0; j < TPL; ++j)
#pragma unroll
                        for (int qq = 0; qq < 8; ++qq) p[j][qq] = 0;
                    // one pair: SELF compares the source with the target's own slot (only the round
                    // that holds the target leaf itself pays for it)
                    auto pairs = [&](auto self_tag) {
                        constexpr bool SELF = decltype(self_tag)::value;
#pragma unroll 1
                        for (int e = 0; e < nj; ++e) {
                            const S4 sx = gx_t[e], sv = gn_t[e];
#pragma unroll
                            for (int j = 0; j < TPL; ++j) {
                                const S rx = sx.x - xs[j][0], ry = sx.y - xs[j][1], rz = sx.z - xs[j][2];
                                S s2 = nb_fma(rx, rx, nb_fma(ry, ry, nb_fma(rz, rz, eps2)));
                                if (GUARD) s2 = s2 > S(0) ? s2 : S(1e30);
                                S inv = GUARD ? nb_rsqrt(s2) : nb_rsqrt_n(s2);
                                if (SELF && e == selfe[j]) inv = S(0);
                                const S inv2 = inv * inv, inv3 = inv2 * inv, inv5 = inv3 * inv2;
                                const S dl = nb_fma(sv.x, rx, nb_fma(sv.y, ry, sv.z * rz));
                                const S dk = nb_fma(nk[j].x, rx, nb_fma(nk[j].y, ry, nk[j].z * rz));
                                const S t = nb_fma(y[j].w, dl, -sx.w * dk) * inv5;
                                p[j][0] = nb_fma(sv.x, inv3, p[j][0]); p[j][1] = nb_fma(sv.y, inv3, p[j][1]);
                                p[j][2] = nb_fma(sv.z, inv3, p[j][2]); p[j][3] = nb_fma(sx.w, inv3, p[j][3]);
                                p[j][4] = nb_fma(rx, t, p[j][4]); p[j][5] = nb_fma(ry, t, p[j][5]);
                                p[j][6] = nb_fma(rz, t, p[j][6]);
                                p[j][7] = nb_fma(dl, inv3, p[j][7]);
                            }
                        }
                    };
                    if (__any_sync(0xffffffffu, self)) pairs(std::true_type());
                    else pairs(std::false_type());
#pragma unroll
                    for (int j = 0; j < TPL; ++j)
#pragma unroll
                        for (int qq = 0; qq < 8; ++qq) {
                            if (KH) kahan_add(sum[j][qq], cmp[j][qq], p[j][qq]);
                            else sum[j][qq] += p[j][qq];
                        }
                    __syncwarp();
                }
            }
        }
        // combine the source groups in a fixed order
        R r[TPL][8];
#pragma unroll
        for (int j = 0; j < TPL; ++j)
#pragma unroll
            for (int qq = 0; qq < 8; ++qq) r[j][qq] = group_sum<MODE>(sum[j][qq], cmp[j][qq], CT);
        if (grp == 0) {
            R* pt = nchunk == 1 ? (R*)A.near + 4 * (int64_t)nt.begin
                                : (R*)A.part + 4 * ((int64_t)A.part_off[li] + (int64_t)chunk * cnt_t);
#pragma unroll
            for (int j = 0; j < TPL; ++j) {
                if (!tv[j]) continue;
                const R qk = (R)y[j].w;
                R* o = pt + 4 * ti[j];
                o[0] = qk * r[j][0] - r[j][3] * (R)nk[j].x - R(3) * r[j][4];
                o[1] = qk * r[j][1] - r[j][3] * (R)nk[j].y - R(3) * r[j][5];
                o[2] = qk * r[j][2] - r[j][3] * (R)nk[j].z - R(3) * r[j][6];
                o[3] = -r[j][7];
            }
        }
        __syncwarp();
    }
}

template <int MODE, int CLS>
__global__ void __launch_bounds__(32 * ADJ_WARPS, AdjShape<CLS>::TPL == 3 ? 3 : 4)
    k_adj_p2p(AdjP2PArgs A, int64_t li_lo, int64_t li_hi, uint32_t w_lo, uint32_t w_hi) {
    typedef typename Prec<MODE>::S4 S4;
    constexpr int CT = AdjShape<CLS>::CT, TPL = AdjShape<CLS>::TPL;
    __shared__ S4 tx[ADJ_WARPS][P2P_WROWS];
    __shared__ S4 tn[ADJ_WARPS][P2P_WROWS];
    const int wib = threadIdx.x >> 5;
    const uint32_t w = w_lo + blockIdx.x * ADJ_WARPS + wib;
    if (w >= w_hi) return;
    const int64_t li = p2p_leaf_of(A.work_off, li_lo, li_hi, w);
    const uint32_t chunk = w - A.work_off[li];
    const uint32_t nchunk = A.work_off[li + 1] - A.work_off[li];
    const uint32_t k = A.leaves[li];
    const NodeRec nt = A.nodes[k];
    const uint32_t lcnt = A.p2p_cnt[k];
    const uint32_t s_lo = chunk * P2P_CHUNK, s_hi = min(lcnt, s_lo + P2P_CHUNK);
    if (A.eps2 > 0.0) adj_item<MODE, false, CT, TPL>(A, tx[wib], tn[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
    else adj_item<MODE, true, CT, TPL>(A, tx[wib], tn[wib], k, nt, li, chunk, nchunk, s_lo, s_hi);
}

// near-field sums of every particle (chunk partials added in chunk order), then the far-field
// adjoint terms and the input-order accumulation; a warp per leaf
template <int MODE, int P>
__global__ void __launch_bounds__(32 * ADJ_WARPS) k_adj_finish(AdjP2PArgs A) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::S S;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    __shared__ S sL[ADJ_WARPS][T];
    __shared__ S sM[ADJ_WARPS][T];
    const int lane = lane_id(), wib = threadIdx.x >> 5;
    const int64_t li = (int64_t)blockIdx.x * ADJ_WARPS + wib;
    if (li >= A.nleaves) return;
    const uint32_t nchunk = A.work_off[li + 1] - A.work_off[li];
    const uint32_t k = A.leaves[li];
    const NodeRec nt = A.nodes[k];
    const H* Lg = (const H*)A.L;
    const H* Mg = (const H*)A.lamM;
    for (int a = lane; a < T; a += 32) {
        sL[wib][a] = (S)Lg[(int64_t)k * T + a];
        sM[wib][a] = (S)Mg[(int64_t)k * T + a];
    }
    __syncwarp();
    const S4* src = (const S4*)A.src;
    const S4* nu = (const S4*)A.nu;
    for (uint32_t ti = lane; ti < nt.count; ti += 32) {
        const uint32_t i = nt.begin + ti;
        R e[4] = {0, 0, 0, 0};
        if (nchunk == 1) {
            const R* pt = (const R*)A.near + 4 * (int64_t)i;
            e[0] = pt[0]; e[1] = pt[1]; e[2] = pt[2]; e[3] = pt[3];
        } else {
            for (uint32_t c = 0; c < nchunk; ++c) {
                const R* pt = (const R*)A.part + 4 * ((int64_t)A.part_off[li] + (int64_t)c * nt.count + ti);
                e[0] += pt[0]; e[1] += pt[1]; e[2] += pt[2]; e[3] += pt[3];
            }
        }
        adj_epilogue<MODE, P>(A, i, sL[wib], sM[wib], src[i], nu[i], e[0], e[1], e[2], e[3]);
    }
}

// host: one VJP at the last evaluated positions; mu = c * lv (input order)
template <int MODE, int P>
int force_vjp(nbody_ctx* c, double coef) {
    typedef typename Prec<MODE>::R R;
    typedef typename Prec<MODE>::H H;
    typedef typename Prec<MODE>::S4 S4;
    constexpr int T = nb_terms<P>::value;
    constexpr int TM = nb_tm<P>::value;
    const int64_t nn = c->nnodes, n = c->n, nl = c->nleaves;
    const int cur = c->cur;
    const BoxDev* box = DP<BoxDev>(c->box);
    NB_TRY(nb_grow(c, c->adj_nu, sizeof(S4) * n));
    NB_TRY(nb_grow(c, c->adj_lamL, sizeof(H) * TM * nn));
    NB_TRY(nb_grow(c, c->adj_lamM, sizeof(H) * T * nn));

    AdjArgs A;
    A.n = n;
    A.ids = DP<uint32_t>(c->id[cur]);
    A.lv = c->adj_lv.p;
    A.q = c->q[cur].p; A.m = c->m[cur].p; A.ax = c->ax[cur].p; A.ay = c->ay[cur].p; A.az = c->az[cur].p;
    A.c = coef;
    A.G = c->prm.G;
    A.nu = c->adj_nu.p;
    A.gx = c->adj_lx.p; A.gq = c->adj_gq.p; A.gm = c->adj_gm.p;
    if (c->timing) cudaEventRecord(c->ev[8], c->st);
    k_adj_prep<MODE><<<(unsigned)((n + 255) / 256), 256, 0, c->st>>>(A);
    NB_LAUNCHED(c, "adj_prep");
    c->launches += 1;
    // near field on the side streams (it needs only the seeds), far-field chain meanwhile on the main one
    AdjP2PArgs C;
    C.leaves = DP<uint32_t>(c->leaves);
    C.nnodes = nn;
    C.n = n;
    C.nleaves = nl;
    C.nodes = DP<NodeRec>(c->nodes);
    C.box = box;
    C.src = c->src.p;
    C.nu = c->adj_nu.p;
    C.L = c->L.p;
    C.lamM = c->adj_lamM.p;
    C.p2p_off = DP<uint32_t>(c->p2p_off); C.p2p_cnt = DP<uint32_t>(c->p2p_cnt); C.p2p_list = DP<uint32_t>(c->p2p_list);
    C.work_off = DP<uint32_t>(c->p2p_work_off);
    C.nwork = (uint32_t)c->h_info[INFO_P2P_WORK];
    C.part_off = DP<uint32_t>(c->p2p_part_off);
    C.part = c->p2p_part.p;
    NB_TRY(nb_grow(c, c->adj_near, 4 * sizeof(R) * (size_t)n));
    C.near = c->adj_near.p;
    C.ids = DP<uint32_t>(c->id[cur]);
    C.gx = c->adj_lx.p;
    C.gq = c->adj_gq.p;
    C.eps2 = c->prm.eps * c->prm.eps;
    {
        const int32_t* hi = c->h_info;
        auto one = [&](auto cls_tag) -> int {
            constexpr int CLS = decltype(cls_tag)::value;
            const uint32_t w0 = (uint32_t)hi[INFO_CLS_WORK + CLS], w1 = (uint32_t)hi[INFO_CLS_WORK + CLS + 1];
            if (w1 <= w0) return NBODY_OK;
            const int64_t l0 = (uint32_t)hi[INFO_CLS_LEAF + CLS], l1 = (uint32_t)hi[INFO_CLS_LEAF + CLS + 1];
            k_adj_p2p<MODE, CLS><<<(w1 - w0 + ADJ_WARPS - 1) / ADJ_WARPS, 32 * ADJ_WARPS, 0, c->side[CLS]>>>(C, l0, l1,
                                                                                                           w0, w1);
            NB_LAUNCHED(c, "adj_p2p");
            c->launches += 1;
            return NBODY_OK;
        };
        NB_TRY(nb_fork(c));
        NB_TRY(one(std::integral_constant<int, 5>()));
        NB_TRY(one(std::integral_constant<int, 4>()));
        NB_TRY(one(std::integral_constant<int, 3>()));
        NB_TRY(one(std::integral_constant<int, 2>()));
        NB_TRY(one(std::integral_constant<int, 1>()));
        NB_TRY(one(std::integral_constant<int, 0>()));
    }
    k_adj_l2pT<MODE, P><<<(unsigned)((nl + 3) / 4), 128, 0, c->st>>>(
        nl, DP<uint32_t>(c->leaves), DP<NodeRec>(c->nodes), DP<S4>(c->src), DP<S4>(c->adj_nu), DP<H>(c->adj_lamL));
    NB_LAUNCHED(c, "adj_l2pT");
    c->launches += 1;
    if (c->timing) cudaEventRecord(c->ev[9], c->st);
    for (int l = c->depth - 1; l >= 0; --l) {
        const int lo = c->level_start[l], hi = c->level_start[l + 1];
        if (hi <= lo) continue;
        k_m2m<MODE, P><<<(unsigned)((hi - lo + 3) / 4), 128, 0, c->st>>>(lo, hi, DP<NodeRec>(c->nodes), box,
                                                                         DP<H>(c->adj_lamL));
        NB_LAUNCHED(c, "adj_l2lT");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[10], c->st);
    {
        M2LArgs B;
        B.nodes = DP<NodeRec>(c->nodes);
        B.box = box;
        B.Mm2l = c->adj_lamL.p;
        B.L = c->adj_lamM.p;
        B.m2l_off = DP<uint32_t>(c->m2l_off); B.m2l_cnt = DP<uint32_t>(c->m2l_cnt);
        B.m2l_list = DP<uint32_t>(c->m2l_list);
        B.eps2 = c->prm.eps * c->prm.eps;
        B.nnodes = nn;
        B.info = DP<int32_t>(c->info);
        B.wait_cycles = c->copy_cycles;
        NB_TRY((dtab_ensure<MODE, P>(c)));
        dtab_args<MODE, P>(c, B);
        constexpr int W = M2LSmem<MODE, P>::warps;
        const size_t smem = (size_t)W * M2LSmem<MODE, P>::per_warp;
        NB_CU(c, cudaFuncSetAttribute(k_m2l<MODE, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        k_m2l<MODE, P><<<(unsigned)((nn + W - 1) / W), 32 * W, smem, c->st>>>(B);
        NB_LAUNCHED(c, "adj_m2lT");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[11], c->st);
    for (int r = 1; r <= c->depth; ++r) {
        const int lo = c->level_start[r], hi = c->level_start[r + 1];
        if (hi <= lo) continue;
        k_l2l<MODE, P><<<(unsigned)((hi - lo + 3) / 4), 128, 0, c->st>>>(lo, hi, DP<NodeRec>(c->nodes), box,
                                                                         DP<H>(c->adj_lamM));
        NB_LAUNCHED(c, "adj_m2mT");
        c->launches += 1;
    }
    if (c->timing) cudaEventRecord(c->ev[12], c->st);
    NB_TRY(nb_join(c));
    k_adj_finish<MODE, P><<<(unsigned)((nl + ADJ_WARPS - 1) / ADJ_WARPS), 32 * ADJ_WARPS, 0, c->st>>>(C);
    NB_LAUNCHED(c, "adj_finish");
    c->launches += 1;
    if (c->timing) cudaEventRecord(c->ev[13], c->st);
    return NBODY_OK;
}

template <int MODE>
int vjp_dispatch(nbody_ctx* c, double coef) {
    switch (c->prm.order) {
        case 1: return force_vjp<MODE, 1>(c, coef);
        case 2: return force_vjp<MODE, 2>(c, coef);
        case 3: return force_vjp<MODE, 3>(c, coef);
        case 4: return force_vjp<MODE, 4>(c, coef);
        case 5: return force_vjp<MODE, 5>(c, coef);
        case 6: return force_vjp<MODE, 6>(c, coef);
        case 7: return force_vjp<MODE, 7>(c, coef);
        case 8: return force_vjp<MODE, 8>(c, coef);
        default: return nb_fail(c, NBODY_ERR_INVALID, "order must be 1..8");
    }
}

}  // namespace nbfmm
