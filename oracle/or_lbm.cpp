// or_lbm.cpp — oracle: D3Q19 BGK collide-stream over an octree of 8^3 bricks.
// TEST INFRASTRUCTURE ONLY (see oracle.h).
//
// The reference generates empty lbm_* kernels (src/parsing/SimulationBuilder.cpp:394-400)
// and keeps D3Q19 only as lattice metadata (include/fluidloom/parsing/LatticeDescriptor.h:15-44),
// so this file is a restatement from the literature, not of reference code
// (parity UNPINNED by the reference):
//  * equilibrium and BGK relaxation: Qian, d'Humieres & Lallemand (1992);
//  * half-way bounce-back and the moving-wall term 6 w_q rho0 (c_q . u_w): Ladd (1994);
//  * equilibrium velocity inlet, zero-gradient outlet (own-site copy): Kruger et al. (2017);
//  * grid refinement with acoustic scaling, tau_l = 2^l (tau_0 - 1/2) + 1/2,
//    level l sub-cycled 2^l times per level-0 step: Dupuis & Chopard (2003),
//    with the coupling done by the reference's own prolongation (copy,
//    split_cells.cl:110-132) and restriction (mean of 8, merge_cells.cl:123-159),
//    applied per population at the interface, and linear interpolation in time
//    of the coarse side for the second fine sub-step.
// All FP32 arithmetic is written operation by operation so the CUDA kernels
// (built without FMA contraction) can reproduce it bit for bit.
#include "oracle.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

namespace {

const uint32_t INV = 0xFFFFFFFFu;
const int Q = 19;
const int CX[Q] = {0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0};
const int CY[Q] = {0, 0, 0, 1, -1, 0, 0, 1, -1, -1, 1, 0, 0, 0, 0, 1, -1, 1, -1};
const int CZ[Q] = {0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, -1, -1, 1, 1, -1, -1, 1};
const int OPP[Q] = {0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17};
// The step's arithmetic is written once for the FP32 oracle (T = float, the
// kernels' operations one by one) and for the FP64 reference run of the same
// steps (T = double) whose difference states the FP32 rounding error.
template <typename T>
inline T wqT(int q) { return q == 0 ? T(1) / T(3) : (q < 7 ? T(1) / T(18) : T(1) / T(36)); }
inline float wq(int q) { return wqT<float>(q); }

// c_q . u as the sum of its non-zero terms in x, y, z order (c = +-1 is a
// sign, so no product is formed; c_0 . u = 0).
template <typename T>
inline T cdotT(int q, T ux, T uy, T uz) {
    const T t[3] = {CX[q] > 0 ? ux : -ux, CY[q] > 0 ? uy : -uy, CZ[q] > 0 ? uz : -uz};
    const int c[3] = {CX[q], CY[q], CZ[q]};
    T s = T(0);
    bool any = false;
    for (int k = 0; k < 3; ++k) {
        if (!c[k]) continue;
        s = any ? s + t[k] : t[k];
        any = true;
    }
    return s;
}
inline float cdot(int q, float ux, float uy, float uz) { return cdotT<float>(q, ux, uy, uz); }

template <typename T>
inline T feqT(int q, T rho, T ux, T uy, T uz, T base) {
    T cu = cdotT<T>(q, ux, uy, uz);
    T t = T(4.5) * cu;
    t = T(3) + t;
    t = cu * t;
    t = base + t;
    T wr = wqT<T>(q) * rho;
    return wr * t;
}
inline float feq1(int q, float rho, float ux, float uy, float uz, float base) {
    return feqT<float>(q, rho, ux, uy, uz, base);
}

template <typename T>
inline T base_ofT(T ux, T uy, T uz) {
    T usq = ux * ux;
    usq = usq + uy * uy;
    usq = usq + uz * uz;
    T t = T(1.5) * usq;
    return T(1) - t;
}
inline float base_of(float ux, float uy, float uz) { return base_ofT<float>(ux, uy, uz); }

// Macroscopic moments in a fixed summation order.
template <typename T>
inline void momentsT(const T* f, T* rho, T* jx, T* jy, T* jz) {
    T r = f[0];
    for (int q = 1; q < Q; ++q) r = r + f[q];
    T a = f[1] - f[2];
    a = a + (f[7] - f[8]); a = a + (f[9] - f[10]); a = a + (f[11] - f[12]); a = a + (f[13] - f[14]);
    T b = f[3] - f[4];
    b = b + (f[7] - f[8]); b = b + (f[10] - f[9]); b = b + (f[15] - f[16]); b = b + (f[17] - f[18]);
    T c = f[5] - f[6];
    c = c + (f[11] - f[12]); c = c + (f[14] - f[13]); c = c + (f[15] - f[16]); c = c + (f[18] - f[17]);
    *rho = r; *jx = a; *jy = b; *jz = c;
}
inline void moments(const float* f, float* rho, float* jx, float* jy, float* jz) { momentsT<float>(f, rho, jx, jy, jz); }

inline int dir_index(int dx, int dy, int dz) {
    int kk = (dz + 1) * 9 + (dy + 1) * 3 + (dx + 1);
    return kk < 13 ? kk : kk - 1;
}

struct CaseInfo {
    int periodic[3];
    float omega[20];
    int mask_level = 0;
    std::vector<uint32_t> mask;  // solid voxels at mask_level, bit (z * Ny + y) * Nx + x; empty: none
};

struct Pool {
    std::vector<or_lbm_case> cases;
    std::vector<CaseInfo> info;
    std::vector<or_domain> doms;
    // bricks
    std::vector<int32_t> x, y, z, flags;
    std::vector<uint8_t> level, state;
    std::vector<uint32_t> mat;
    std::vector<uint16_t> cs;
    std::vector<uint32_t> nbr;
    std::vector<float> f[2];
    size_t n = 0;
    int maxL = 0;
    int parity[20] = {0};
    or_mesh mesh() {
        or_mesh m;
        m.x = x.data(); m.y = y.data(); m.z = z.data(); m.level = level.data(); m.state = state.data();
        m.flags = flags.data(); m.material = mat.data(); m.case_id = cs.data(); m.n = n;
        return m;
    }
};

inline size_t fidx(size_t n, int q, size_t b, int s) { return ((size_t)q * n + b) * 512 + s; }

// Mask voxel under the centre of level-l site (sx, sy, sz): a coarser site
// samples the voxel at its centre (the upper of the two middle ones), a finer
// site the voxel holding it; sites outside the case grid are fluid.
inline bool mask_at(const or_lbm_case& c, const CaseInfo& ci, int64_t sx, int64_t sy, int64_t sz, int l) {
    const int64_t G[3] = {sx, sy, sz};
    int64_t v[3], N[3];
    const int sh = ci.mask_level - l;
    for (int a = 0; a < 3; ++a) {
        if (G[a] < 0 || G[a] >= ((int64_t)c.ext[a] * 8 << l)) return false;
        N[a] = (int64_t)c.ext[a] * 8 << ci.mask_level;
        if (sh >= 0) v[a] = G[a] * ((int64_t)1 << sh) + (sh > 0 ? (int64_t)1 << (sh - 1) : 0);
        else v[a] = G[a] / ((int64_t)1 << -sh);
    }
    const uint64_t i = ((uint64_t)v[2] * (uint64_t)N[1] + (uint64_t)v[1]) * (uint64_t)N[0] + (uint64_t)v[0];
    return (ci.mask[i >> 5] >> (i & 31)) & 1u;
}

// Solid: inside the case's sphere or on a voxel of its solid mask.
inline bool solid_at(const or_lbm_case& c, const CaseInfo& ci, int64_t sx, int64_t sy, int64_t sz, int l) {
    if (c.has_sphere) {
        float inv = 1.0f / (float)(1 << l);
        float px = ((float)sx + 0.5f) * inv, py = ((float)sy + 0.5f) * inv, pz = ((float)sz + 0.5f) * inv;
        float dx = px - c.sphere_c[0], dy = py - c.sphere_c[1], dz = pz - c.sphere_c[2];
        float d2 = dx * dx;
        d2 = d2 + dy * dy;
        d2 = d2 + dz * dz;
        float r2 = c.sphere_r * c.sphere_r;
        if (d2 < r2) return true;
    }
    return !ci.mask.empty() && mask_at(c, ci, sx, sy, sz, l);
}

// Pull of population q into site G (global level-l coords) of brick b; F =
// the two population buffers (of type T), R = level l's current one.
template <typename T>
T pullT(const Pool& P, const std::vector<T>* F, size_t b, int q, int l, int sub, const int64_t* G, const T* R) {
    const or_lbm_case& c = P.cases[P.cs[b]];
    const CaseInfo& ci = P.info[P.cs[b]];
    int64_t S[3] = {G[0] - CX[q], G[1] - CY[q], G[2] - CZ[q]};
    int64_t N[3];
    for (int a = 0; a < 3; ++a) N[a] = (int64_t)c.ext[a] * 8 << l;
    int out_face[3] = {-1, -1, -1};
    bool out = false;
    for (int a = 0; a < 3; ++a) {
        if (ci.periodic[a]) continue;
        if (S[a] < 0) { out_face[a] = 2 * a; out = true; }
        else if (S[a] >= N[a]) { out_face[a] = 2 * a + 1; out = true; }
    }
    int s_local = (int)((G[0] - (int64_t)P.x[b] * 8) + 8 * (G[1] - (int64_t)P.y[b] * 8) + 64 * (G[2] - (int64_t)P.z[b] * 8));
    if (out) {
        bool inlet = false, outlet = false;
        int moving = -1;
        for (int a = 0; a < 3; ++a) {
            if (out_face[a] < 0) continue;
            int bt = c.bc[out_face[a]];
            if (bt == 3) inlet = true;
            else if (bt == 4) outlet = true;
            else if (bt == 2 && moving < 0) moving = out_face[a];
        }
        if (inlet) {
            const T iu[3] = {T(c.inlet_u[0]), T(c.inlet_u[1]), T(c.inlet_u[2])};
            T base = base_ofT<T>(iu[0], iu[1], iu[2]);
            return feqT<T>(q, T(1), iu[0], iu[1], iu[2], base);
        }
        if (outlet) return R[fidx(P.n, q, b, s_local)];
        T v = R[fidx(P.n, OPP[q], b, s_local)];
        if (moving >= 0) {
            T cu = cdotT<T>(q, T(c.wall_u[0]), T(c.wall_u[1]), T(c.wall_u[2]));
            T t = T(6) * wqT<T>(q);
            t = t * cu;
            v = v + t;
        }
        return v;
    }
    int64_t Sw[3];
    for (int a = 0; a < 3; ++a) Sw[a] = ci.periodic[a] ? ((S[a] % N[a]) + N[a]) % N[a] : S[a];
    if (solid_at(c, ci, Sw[0], Sw[1], Sw[2], l)) return R[fidx(P.n, OPP[q], b, s_local)];
    // local coordinates of the (unwrapped) source relative to brick b
    int64_t L[3] = {S[0] - (int64_t)P.x[b] * 8, S[1] - (int64_t)P.y[b] * 8, S[2] - (int64_t)P.z[b] * 8};
    if (L[0] >= 0 && L[0] < 8 && L[1] >= 0 && L[1] < 8 && L[2] >= 0 && L[2] < 8)
        return R[fidx(P.n, q, b, (int)(L[0] + 8 * L[1] + 64 * L[2]))];
    int d[3], sub_slot = 0, bit = 0;
    for (int a = 0; a < 3; ++a) {
        d[a] = L[a] < 0 ? -1 : (L[a] >= 8 ? 1 : 0);
        if (d[a] == 0) { if (L[a] >= 4) sub_slot |= 1 << bit; ++bit; }
    }
    uint32_t nb = P.nbr[(b * 26 + dir_index(d[0], d[1], d[2])) * 4 + sub_slot];
    if (nb == INV) return R[fidx(P.n, OPP[q], b, s_local)];
    int ln = P.level[nb];
    if (ln == l) {
        int64_t lx = Sw[0] - (int64_t)P.x[nb] * 8, ly = Sw[1] - (int64_t)P.y[nb] * 8, lz = Sw[2] - (int64_t)P.z[nb] * 8;
        return R[fidx(P.n, q, nb, (int)(lx + 8 * ly + 64 * lz))];
    }
    if (ln == l - 1) {
        int64_t lx = (Sw[0] >> 1) - (int64_t)P.x[nb] * 8, ly = (Sw[1] >> 1) - (int64_t)P.y[nb] * 8,
                lz = (Sw[2] >> 1) - (int64_t)P.z[nb] * 8;
        size_t i = fidx(P.n, q, nb, (int)(lx + 8 * ly + 64 * lz));
        const T* oldb = F[1 - P.parity[l - 1]].data();
        const T* newb = F[P.parity[l - 1]].data();
        if (sub == 0) return oldb[i];
        T t = oldb[i] + newb[i];
        return t * T(0.5);
    }
    if (ln == l + 1) {
        const T* fb = F[P.parity[l + 1]].data();
        T s = T(0);
        for (int k = 0; k < 8; ++k) {
            int64_t lx = 2 * Sw[0] + (k & 1) - (int64_t)P.x[nb] * 8;
            int64_t ly = 2 * Sw[1] + ((k >> 1) & 1) - (int64_t)P.y[nb] * 8;
            int64_t lz = 2 * Sw[2] + ((k >> 2) & 1) - (int64_t)P.z[nb] * 8;
            s = s + fb[fidx(P.n, q, nb, (int)(lx + 8 * ly + 64 * lz))];
        }
        return s * T(0.125);
    }
    return R[fidx(P.n, OPP[q], b, s_local)];
}

// omega(case, l) gives the relaxation rate in T.
template <typename T, typename Omega>
void collide_streamT(Pool& P, std::vector<T>* F, Omega omega_of, int l, int sub, int nthreads) {
    const T* R = F[P.parity[l]].data();
    T* Wt = F[1 - P.parity[l]].data();
    long long nb = (long long)P.n;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads)
    for (long long b = 0; b < nb; ++b) {
        if (P.level[b] != l) continue;
        const or_lbm_case& c = P.cases[P.cs[b]];
        const CaseInfo& ci = P.info[P.cs[b]];
        const T omega = omega_of(P.cs[b], l);
        for (int s = 0; s < 512; ++s) {
            int64_t G[3] = {(int64_t)P.x[b] * 8 + (s & 7), (int64_t)P.y[b] * 8 + ((s >> 3) & 7),
                            (int64_t)P.z[b] * 8 + (s >> 6)};
            if (solid_at(c, ci, G[0], G[1], G[2], l)) {
                for (int q = 0; q < Q; ++q) Wt[fidx(P.n, q, b, s)] = wqT<T>(q);
                continue;
            }
            T fin[Q];
            for (int q = 0; q < Q; ++q) fin[q] = pullT<T>(P, F, b, q, l, sub, G, R);
            T rho, jx, jy, jz;
            momentsT<T>(fin, &rho, &jx, &jy, &jz);
            T inv = T(1) / rho;
            T ux = jx * inv, uy = jy * inv, uz = jz * inv;
            T base = base_ofT<T>(ux, uy, uz);
            for (int q = 0; q < Q; ++q) {
                T fe = feqT<T>(q, rho, ux, uy, uz, base);
                T d = fe - fin[q];
                d = omega * d;
                Wt[fidx(P.n, q, b, s)] = fin[q] + d;
            }
        }
    }
    P.parity[l] ^= 1;
}

template <typename T, typename Omega>
void step_levelT(Pool& P, std::vector<T>* F, Omega omega_of, int l, int sub, int nthreads) {
    collide_streamT<T>(P, F, omega_of, l, sub, nthreads);
    if (l < P.maxL) {
        step_levelT<T>(P, F, omega_of, l + 1, 0, nthreads);
        step_levelT<T>(P, F, omega_of, l + 1, 1, nthreads);
    }
}

void step_level(Pool& P, int l, int sub, int nthreads) {
    step_levelT<float>(P, P.f, [&P](int cs, int lv) { return P.info[cs].omega[lv]; }, l, sub, nthreads);
}

void derive(Pool& P) {
    P.info.resize(P.cases.size());
    P.doms.resize(P.cases.size());
    P.maxL = 0;
    for (size_t i = 0; i < P.cases.size(); ++i) {
        const or_lbm_case& c = P.cases[i];
        for (int a = 0; a < 3; ++a) P.info[i].periodic[a] = c.bc[2 * a] == 0;
        for (int l = 0; l < 20; ++l) {
            float t = c.tau0 - 0.5f;
            t = (float)(1 << l) * t;
            t = t + 0.5f;
            P.info[i].omega[l] = 1.0f / t;
        }
        or_domain& d = P.doms[i];
        d.depth = 17; d.anchor_level = 13; d.max_level = 13;
        for (int a = 0; a < 3; ++a) { d.ext[a] = c.ext[a]; d.periodic[a] = P.info[i].periodic[a]; }
        P.maxL = std::max(P.maxL, (int)c.max_level);
    }
}

void rebuild_nbr(Pool& P) {
    P.nbr.assign(P.n * 26 * 4, INV);
    or_mesh m = P.mesh();
    or_neighbours(&m, P.doms.data(), 4, P.nbr.data());
}

// Geometric band test of a brick against the sphere (FP32, fixed order).
bool in_band(const or_lbm_case& c, int32_t bx, int32_t by, int32_t bz, int l) {
    if (!c.has_sphere) return false;
    float inv = 1.0f / (float)(1 << l);
    int32_t nat[3] = {bx, by, bz};
    float dmin = 0.0f, dmax = 0.0f;
    for (int a = 0; a < 3; ++a) {
        float lo = (float)(nat[a] * 8) * inv;
        float hi = (float)(nat[a] * 8 + 8) * inv;
        float cc = c.sphere_c[a];
        float cl = cc < lo ? lo : (cc > hi ? hi : cc);
        float e = cc - cl;
        dmin = dmin + e * e;
        float f1 = std::fabs(cc - lo), f2 = std::fabs(cc - hi);
        float fm = f1 > f2 ? f1 : f2;
        dmax = dmax + fm * fm;
    }
    float ro = c.sphere_r + c.band;
    float ri = c.sphere_r - c.band;
    if (ri < 0.0f) ri = 0.0f;
    return dmin <= ro * ro && dmax >= ri * ri;
}

// Velocity of a site from its populations (fixed order), 0 in solid sites.
inline void site_u(const Pool& P, const float* F, size_t b, int s, int l, float* u) {
    const or_lbm_case& c = P.cases[P.cs[b]];
    int64_t G[3] = {(int64_t)P.x[b] * 8 + (s & 7), (int64_t)P.y[b] * 8 + ((s >> 3) & 7), (int64_t)P.z[b] * 8 + (s >> 6)};
    if (solid_at(c, P.info[P.cs[b]], G[0], G[1], G[2], l)) { u[0] = u[1] = u[2] = 0.0f; return; }
    float f[Q];
    for (int q = 0; q < Q; ++q) f[q] = F[fidx(P.n, q, b, s)];
    float rho, jx, jy, jz;
    moments(f, &rho, &jx, &jy, &jz);
    float inv = 1.0f / rho;
    u[0] = jx * inv; u[1] = jy * inv; u[2] = jz * inv;
}

void brick_vorticity(const Pool& P, size_t b, float* wmax) {
    int l = P.level[b];
    const float* F = P.f[P.parity[l]].data();
    static thread_local float U[512][3];
    for (int s = 0; s < 512; ++s) site_u(P, F, b, s, l, U[s]);
    float scale = (float)(1 << l);
    float m = 0.0f;
    for (int s = 0; s < 512; ++s) {
        int i = s & 7, j = (s >> 3) & 7, k = s >> 6;
        auto d = [&](int comp, int axis) {
            int co[3] = {i, j, k};
            int stride = axis == 0 ? 1 : (axis == 1 ? 8 : 64);
            if (co[axis] == 0) return U[s + stride][comp] - U[s][comp];
            if (co[axis] == 7) return U[s][comp] - U[s - stride][comp];
            float t = U[s + stride][comp] - U[s - stride][comp];
            return t * 0.5f;
        };
        float wx = d(2, 1) - d(1, 2);
        float wy = d(0, 2) - d(2, 0);
        float wz = d(1, 0) - d(0, 1);
        float w2 = wx * wx;
        w2 = w2 + wy * wy;
        w2 = w2 + wz * wz;
        float mag = std::sqrt(w2) * scale;
        m = mag > m ? mag : m;
    }
    *wmax = m;
}

// A brick of a masked case whose own sites and one-site halo (periodic axes
// wrapped) hold both solid and fluid sites: some halo site solid, not all own
// sites solid.
bool mask_mixed(const Pool& P, size_t b) {
    const or_lbm_case& c = P.cases[P.cs[b]];
    const CaseInfo& ci = P.info[P.cs[b]];
    if (ci.mask.empty()) return false;
    const int l = P.level[b];
    const int64_t G0[3] = {(int64_t)P.x[b] * 8, (int64_t)P.y[b] * 8, (int64_t)P.z[b] * 8};
    bool any = false, all = true;
    for (int i = 0; i < 1000; ++i) {
        const int h[3] = {i % 10, (i / 10) % 10, i / 100};
        int64_t G[3];
        for (int a = 0; a < 3; ++a) {
            G[a] = G0[a] + h[a] - 1;
            if (!ci.periodic[a]) continue;
            const int64_t N = ((int64_t)c.ext[a] * 8) << l;
            G[a] = G[a] < 0 ? G[a] + N : (G[a] >= N ? G[a] - N : G[a]);
        }
        const bool sol = solid_at(c, ci, G[0], G[1], G[2], l);
        const bool own = h[0] >= 1 && h[0] <= 8 && h[1] >= 1 && h[1] <= 8 && h[2] >= 1 && h[2] <= 8;
        any = any || sol;
        all = all && (sol || !own);
    }
    return any && !all;
}

void compute_flags(Pool& P, bool use_vorticity, float* out_wmax) {
    std::vector<float> wm(P.n, 0.0f);
    if (use_vorticity) {
#pragma omp parallel for schedule(dynamic, 4)
        for (long long b = 0; b < (long long)P.n; ++b) brick_vorticity(P, b, &wm[b]);
    }
    std::vector<float> cmax(P.cases.size(), 0.0f);
    for (size_t b = 0; b < P.n; ++b) cmax[P.cs[b]] = wm[b] > cmax[P.cs[b]] ? wm[b] : cmax[P.cs[b]];
    for (size_t b = 0; b < P.n; ++b) {
        const or_lbm_case& c = P.cases[P.cs[b]];
        int l = P.level[b];
        bool band = in_band(c, P.x[b], P.y[b], P.z[b], l) || mask_mixed(P, b);
        float cm = cmax[P.cs[b]];
        int32_t fl = 0;
        if (band) fl = l < c.max_level ? 1 : 0;
        else if (cm > 0.0f && wm[b] > c.refine_frac * cm && l < c.max_level) fl = 1;
        else if (wm[b] < c.coarsen_frac * cm && l > 0) fl = -1;
        P.flags[b] = fl;
        if (out_wmax) out_wmax[b] = wm[b];
    }
}

// One regrid of the pool: adapt with FULL26 balance, then remap populations:
// survivors copied, children take the parent site covering them (copy),
// parents take the mean of the 2x2x2 child sites (children 0..7 in bit order).
void regrid_with_flags(Pool& P);

void regrid(Pool& P, bool use_vorticity) {
    compute_flags(P, use_vorticity, nullptr);
    regrid_with_flags(P);
}

void regrid_with_flags(Pool& P) {
    or_mesh m = P.mesh();
    or_adapt_cfg cfg{P.maxL, 0, 1, 10, 1, 0};
    size_t cap = P.n * 8 + 8;
    std::vector<int32_t> ox(cap), oy(cap), oz(cap), ofl(cap);
    std::vector<uint8_t> ol(cap), os(cap), okind(cap);
    std::vector<uint32_t> om(cap), osrc(cap), omem(cap);
    std::vector<uint16_t> oc(cap);
    or_adapt_stats st;
    size_t M = or_adapt(&m, P.doms.data(), &cfg, nullptr, 0, 0, ox.data(), oy.data(), oz.data(), ol.data(),
                        os.data(), ofl.data(), om.data(), oc.data(), nullptr, osrc.data(), okind.data(),
                        omem.data(), &st);
    std::vector<float> nf((size_t)Q * M * 512);
    size_t on = P.n;
    for (size_t j = 0; j < M; ++j) {
        int kind = okind[j];
        for (int s = 0; s < 512; ++s) {
            int I = s & 7, J = (s >> 3) & 7, K = s >> 6;
            for (int q = 0; q < Q; ++q) {
                float v;
                if (kind == 8) {
                    const float* F = P.f[P.parity[P.level[osrc[j]]]].data();
                    v = F[fidx(on, q, osrc[j], s)];
                } else if (kind < 8) {
                    uint32_t pb = osrc[j];
                    const float* F = P.f[P.parity[P.level[pb]]].data();
                    int ps = (4 * (kind & 1) + I / 2) + 8 * (4 * ((kind >> 1) & 1) + J / 2) + 64 * (4 * ((kind >> 2) & 1) + K / 2);
                    v = F[fidx(on, q, pb, ps)];
                } else {
                    int oc8 = (I >> 2) | ((J >> 2) << 1) | ((K >> 2) << 2);
                    uint32_t cb = omem[(size_t)osrc[j] * 8 + oc8];
                    const float* F = P.f[P.parity[P.level[cb]]].data();
                    float sum = 0.0f;
                    for (int t = 0; t < 8; ++t) {
                        int fs = (2 * (I & 3) + (t & 1)) + 8 * (2 * (J & 3) + ((t >> 1) & 1)) + 64 * (2 * (K & 3) + ((t >> 2) & 1));
                        sum = sum + F[fidx(on, q, cb, fs)];
                    }
                    v = sum * 0.125f;
                }
                nf[fidx(M, q, j, s)] = v;
            }
        }
    }
    P.x.assign(ox.begin(), ox.begin() + M); P.y.assign(oy.begin(), oy.begin() + M); P.z.assign(oz.begin(), oz.begin() + M);
    P.level.assign(ol.begin(), ol.begin() + M); P.state.assign(os.begin(), os.begin() + M);
    P.flags.assign(M, 0); P.mat.assign(om.begin(), om.begin() + M); P.cs.assign(oc.begin(), oc.begin() + M);
    P.n = M;
    P.f[0].swap(nf);
    P.f[1].assign((size_t)Q * M * 512, 0.0f);
    for (int l = 0; l < 20; ++l) P.parity[l] = 0;
    rebuild_nbr(P);
}

void init_populations(Pool& P) {
    P.f[0].assign((size_t)Q * P.n * 512, 0.0f);
    P.f[1].assign((size_t)Q * P.n * 512, 0.0f);
    for (size_t b = 0; b < P.n; ++b) {
        const or_lbm_case& c = P.cases[P.cs[b]];
        float base = base_of(c.init_u[0], c.init_u[1], c.init_u[2]);
        for (int q = 0; q < Q; ++q) {
            float v = feq1(q, 1.0f, c.init_u[0], c.init_u[1], c.init_u[2], base);
            for (int s = 0; s < 512; ++s) P.f[0][fidx(P.n, q, b, s)] = v;
        }
    }
    for (int l = 0; l < 20; ++l) P.parity[l] = 0;
}

}  // namespace

// exp(x) for x <= 0: Cody & Waite (1980) reduction x = n ln2 + r with ln2
// split into a 16-bit head (0.693145751953125, so n*head is exact) and a tail
// (the split published with fdlibm's single-precision expf, e_expf.c), Taylor
// series of e^r to r^7, exact scaling by 2^n.  Operation by operation, as the
// CUDA flag kernel computes it.
static float exp_neg(float x) {
    if (x < -87.0f) return 0.0f;
    float t = x * 1.44269504f;
    t = t + 0.5f;
    float n = std::floor(t);
    float r = x - n * 0.693145752f;
    r = r - n * 1.42860677e-06f;
    float p = 1.0f / 5040.0f;
    p = p * r; p = p + 1.0f / 720.0f;
    p = p * r; p = p + 1.0f / 120.0f;
    p = p * r; p = p + 1.0f / 24.0f;
    p = p * r; p = p + 1.0f / 6.0f;
    p = p * r; p = p + 0.5f;
    p = p * r; p = p + 1.0f;
    p = p * r; p = p + 1.0f;
    return std::ldexp(p, (int)n);
}

extern "C" {

// Flags from a sum of Gaussian blobs {cx, cy, cz, 1/(2 sigma^2), amplitude}
// at cell centres (native + 0.5) / 2^level: 1 above hi (below max level),
// -1 below lo.
void or_blob_flags(const int32_t* x, const int32_t* y, const int32_t* z, const uint8_t* level, size_t n,
                   const float* blobs, int nblobs, float lo, float hi, int max_level, int32_t* flags) {
#pragma omp parallel for schedule(static)
    for (long long i = 0; i < (long long)n; ++i) {
        int l = level[i];
        float inv = 1.0f / (float)(1 << l);
        float px = ((float)x[i] + 0.5f) * inv, py = ((float)y[i] + 0.5f) * inv, pz = ((float)z[i] + 0.5f) * inv;
        float v = 0.0f;
        for (int k = 0; k < nblobs; ++k) {
            const float* B = blobs + 5 * k;
            float dx = px - B[0], dy = py - B[1], dz = pz - B[2];
            float d2 = dx * dx;
            d2 = d2 + dy * dy;
            d2 = d2 + dz * dz;
            float e = exp_neg(-(d2 * B[3]));
            v = v + B[4] * e;
        }
        int32_t f = 0;
        if (v > hi && l < max_level) f = 1;
        else if (v < lo) f = -1;
        flags[i] = f;
    }
}

// Build a pool: per case, level-0 bricks covering ext, then max_level rounds of
// band-only refinement (adapt with FULL26 balance), then equilibrium
// populations at rho = 1, u = init_u.
void* or_pool_new(const or_lbm_case* cases, int ncases) {
    Pool* P = new Pool();
    P->cases.assign(cases, cases + ncases);
    derive(*P);
    for (int ci = 0; ci < ncases; ++ci) {
        const or_lbm_case& c = cases[ci];
        for (int32_t k = 0; k < c.ext[2]; ++k)
            for (int32_t j = 0; j < c.ext[1]; ++j)
                for (int32_t i = 0; i < c.ext[0]; ++i) {
                    P->x.push_back(i); P->y.push_back(j); P->z.push_back(k);
                    P->level.push_back(0); P->state.push_back(0); P->flags.push_back(0);
                    P->mat.push_back(0); P->cs.push_back((uint16_t)ci);
                }
    }
    P->n = P->x.size();
    // order by key once so that the pool starts sorted
    {
        std::vector<uint64_t> k(P->n);
        std::vector<uint32_t> id(P->n);
        or_cell_keys(P->x.data(), P->y.data(), P->z.data(), P->level.data(), P->cs.data(), 17, 13, k.data(), P->n);
        for (size_t i = 0; i < P->n; ++i) id[i] = (uint32_t)i;
        or_sort_pairs_u64_u32(k.data(), id.data(), P->n);
        Pool T = *P;
        for (size_t i = 0; i < P->n; ++i) {
            P->x[i] = T.x[id[i]]; P->y[i] = T.y[id[i]]; P->z[i] = T.z[id[i]]; P->cs[i] = T.cs[id[i]];
        }
    }
    rebuild_nbr(*P);
    init_populations(*P);
    for (int r = 0; r < P->maxL; ++r) regrid(*P, false);
    init_populations(*P);
    return P;
}

void or_pool_free(void* h) { delete (Pool*)h; }

// The case's solid mask (fl_pool_set_solid_mask): bits == NULL removes it.
void or_pool_set_mask(void* h, int case_id, int level, const uint32_t* bits, size_t nwords) {
    Pool& P = *(Pool*)h;
    CaseInfo& ci = P.info[case_id];
    ci.mask_level = bits ? level : 0;
    ci.mask.assign(bits, bits ? bits + nwords : bits);
}

void or_pool_steps(void* h, int nsteps, int nthreads) {
    Pool& P = *(Pool*)h;
    for (int i = 0; i < nsteps; ++i) step_level(P, 0, 0, nthreads);
}

// The pool's next nsteps level-0 steps in FP64 from its current (FP32) state,
// on its current mesh; the pool itself is left as it is.  out: the resulting
// populations as or_pool_populations lays them out, in double.
void or_pool_fp64_steps(void* h, int nsteps, int nthreads, double* out) {
    const Pool& P0 = *(const Pool*)h;
    Pool P = P0;
    std::vector<double> F[2];
    for (int k = 0; k < 2; ++k) F[k].assign(P0.f[k].begin(), P0.f[k].end());
    std::vector<double> omega(P.cases.size() * 20);
    for (size_t c = 0; c < P.cases.size(); ++c)
        for (int l = 0; l < 20; ++l) {
            double t = (double)P.cases[c].tau0 - 0.5;
            t = (double)(1 << l) * t;
            t = t + 0.5;
            omega[c * 20 + l] = 1.0 / t;
        }
    auto omega_of = [&omega](int cs, int l) { return omega[(size_t)cs * 20 + l]; };
    for (int i = 0; i < nsteps; ++i) step_levelT<double>(P, F, omega_of, 0, 0, nthreads);
    for (size_t b = 0; b < P.n; ++b) {
        const double* G = F[P.parity[P.level[b]]].data();
        for (int q = 0; q < Q; ++q) std::memcpy(out + fidx(P.n, q, b, 0), G + fidx(P.n, q, b, 0), 512 * 8);
    }
}

void or_pool_regrid(void* h) { regrid(*(Pool*)h, true); }

// A regrid with the caller's flags (one per brick, pool order: > 0 split,
// -1 merge, 0 keep), as fl_pool_regrid_flags.
void or_pool_regrid_flags(void* h, const int32_t* flags) {
    Pool& P = *(Pool*)h;
    std::memcpy(P.flags.data(), flags, P.n * 4);
    regrid_with_flags(P);
}

// Replace the populations of every brick ([19][n][512], pool order), all
// levels at parity 0, as fl_pool_upload.
void or_pool_upload(void* h, const float* f) {
    Pool& P = *(Pool*)h;
    std::memcpy(P.f[0].data(), f, sizeof(float) * (size_t)Q * P.n * 512);
    for (int l = 0; l < 20; ++l) P.parity[l] = 0;
}

void or_pool_flags(void* h, int32_t* flags, float* wmax) {
    Pool& P = *(Pool*)h;
    compute_flags(P, true, wmax);
    if (flags) std::memcpy(flags, P.flags.data(), P.n * 4);
}

size_t or_pool_size(void* h) { return ((Pool*)h)->n; }

void or_pool_bricks(void* h, int32_t* x, int32_t* y, int32_t* z, uint8_t* level, uint16_t* cs) {
    Pool& P = *(Pool*)h;
    for (size_t i = 0; i < P.n; ++i) {
        x[i] = P.x[i]; y[i] = P.y[i]; z[i] = P.z[i]; level[i] = P.level[i]; cs[i] = P.cs[i];
    }
}

void or_pool_nbr(void* h, uint32_t* out) {
    Pool& P = *(Pool*)h;
    std::memcpy(out, P.nbr.data(), P.nbr.size() * 4);
}

// Current populations of every brick ([19][n][512], each brick from its level's buffer).
void or_pool_populations(void* h, float* out) {
    Pool& P = *(Pool*)h;
    for (size_t b = 0; b < P.n; ++b) {
        const float* F = P.f[P.parity[P.level[b]]].data();
        for (int q = 0; q < Q; ++q) std::memcpy(out + fidx(P.n, q, b, 0), F + fidx(P.n, q, b, 0), 512 * 4);
    }
}

// Per case: fluid mass and momentum, each site weighted by its volume 8^-level,
// summed in FP64 in brick order.
void or_pool_conservation(void* h, double* out) {
    Pool& P = *(Pool*)h;
    std::memset(out, 0, sizeof(double) * 4 * P.cases.size());
    for (size_t b = 0; b < P.n; ++b) {
        int l = P.level[b];
        const float* F = P.f[P.parity[l]].data();
        const or_lbm_case& c = P.cases[P.cs[b]];
        double vol = 1.0 / (double)(1ull << (3 * l));
        double acc[4] = {0, 0, 0, 0};
        for (int s = 0; s < 512; ++s) {
            int64_t G[3] = {(int64_t)P.x[b] * 8 + (s & 7), (int64_t)P.y[b] * 8 + ((s >> 3) & 7), (int64_t)P.z[b] * 8 + (s >> 6)};
            if (solid_at(c, P.info[P.cs[b]], G[0], G[1], G[2], l)) continue;
            float f[Q];
            for (int q = 0; q < Q; ++q) f[q] = F[fidx(P.n, q, b, s)];
            float rho, jx, jy, jz;
            moments(f, &rho, &jx, &jy, &jz);
            acc[0] += rho; acc[1] += jx; acc[2] += jy; acc[3] += jz;
        }
        for (int k = 0; k < 4; ++k) out[4 * P.cs[b] + k] += acc[k] * vol;
    }
}

// Fluid site updates per level-0 step: sum over fluid sites of 2^level.
uint64_t or_pool_fluid_lups(void* h) {
    Pool& P = *(Pool*)h;
    uint64_t t = 0;
    for (size_t b = 0; b < P.n; ++b) {
        int l = P.level[b];
        const or_lbm_case& c = P.cases[P.cs[b]];
        uint64_t cnt = 0;
        for (int s = 0; s < 512; ++s) {
            int64_t G[3] = {(int64_t)P.x[b] * 8 + (s & 7), (int64_t)P.y[b] * 8 + ((s >> 3) & 7), (int64_t)P.z[b] * 8 + (s >> 6)};
            if (!solid_at(c, P.info[P.cs[b]], G[0], G[1], G[2], l)) ++cnt;
        }
        t += cnt << l;
    }
    return t;
}

}  // extern "C"
