// ct_adjoint.cu -- reverse-mode derivatives (no upstream counterpart) of two
// upstream float64 functions, with the intersection indices held fixed:
//
//   * the area of intersection of a subject face clipped by a tree face:
//     polygon_polygon_clip_area (algorithms/sutherland_hodgman.py:83-148)
//     followed by polygon_area (geometry_utils.py:82-95, a fan of |cross|);
//   * the barycentric weights of a point in a tree face:
//     barycentric_triangle.py:28-43 and barycentric_wachspress.py:26-85
//     (including the on-edge linear interpolation branch).
//
// Each kernel replays the forward computation in the same order (so it takes
// the same branches as the forward kernels and upstream), then propagates the
// upstream gradient backwards and scatters it into per-vertex gradients with
// float64 atomics (summation order, hence the last bits, vary between runs).
// Points where the function is not differentiable (a vertex exactly on a clip
// line, |cross| = 0) take the subgradient that treats sign(0) as 0.
#include <cstdint>

#include "ct_common.cuh"
#include "ct_geom.cuh"
#include "ct_internal.h"

namespace cta {

constexpr int TAPE_MAX = 160;  // subject vertices + intersection nodes per pair

__device__ __forceinline__ double sgn(double x) { return (x > 0.0) ? 1.0 : ((x < 0.0) ? -1.0 : 0.0); }

__device__ __forceinline__ void acc(dpt* a, double gx, double gy) {
    a->x += gx;
    a->y += gy;
}

// Sutherland-Hodgman clip (subject = polygon a, clipper = polygon b) with a
// tape: node k < la is subject vertex k; a later node is the intersection of
// the segment from node pa to node pb with the line through clipper vertices
// pr -> ps.  Returns the number of nodes, the final polygon in `cur` (node
// ids) and its length; -1 when the tape or a scratch polygon would overflow.
struct Clip {
    dpt P[TAPE_MAX];
    short pa[TAPE_MAX], pb[TAPE_MAX];
    unsigned char pr[TAPE_MAX], ps[TAPE_MAX];
    short bufA[CT_CLIP_MAX], bufB[CT_CLIP_MAX];
};

__device__ int clip_taped(Clip& C, const dpt* subj, int la, const dpt* clip, int lb, short** cur_out, int* ncur_out) {
    int nn = 0;
    for (int k = 0; k < la; k++) C.P[nn++] = subj[k];
    short* output = C.bufA;
    short* subject = C.bufB;
    int n_output = la;
    for (int k = 0; k < la; k++) output[k] = (short)k;
    int ir = lb - 1;
    dpt r = clip[ir];
    for (int i = 0; i < lb; i++) {
        dpt s = clip[i];
        dpt U = mkp(s.x - r.x, s.y - r.y);
        if (U.x == 0 && U.y == 0) continue;
        dpt N = mkp(-U.y, U.x);
        int length = n_output;
        short* t = subject;
        subject = output;
        output = t;
        n_output = 0;
        short ia = subject[length - 1];
        bool a_inside = sh_inside(C.P[ia], r, U);
        for (int j = 0; j < length; j++) {
            short ib = subject[j];
            dpt a = C.P[ia], b = C.P[ib];
            dpt V = mkp(b.x - a.x, b.y - a.y);
            if (V.x == 0 && V.y == 0) continue;
            bool b_inside = sh_inside(b, r, U);
            dpt pnt;
            bool push_isect = false, push_b = false;
            if (b_inside) {
                if (!a_inside) push_isect = sh_intersection(a, V, r, N, &pnt);
                push_b = true;
            } else if (a_inside) {
                if (sh_intersection(a, V, r, N, &pnt)) {
                    push_isect = true;
                } else {
                    b_inside = true;
                    push_b = true;
                }
            }
            if (push_isect) {
                if (nn >= TAPE_MAX || n_output >= CT_CLIP_MAX) return -1;
                C.P[nn] = pnt;
                C.pa[nn] = ia;
                C.pb[nn] = ib;
                C.pr[nn] = (unsigned char)ir;
                C.ps[nn] = (unsigned char)i;
                output[n_output++] = (short)nn;
                nn++;
            }
            if (push_b) {
                if (n_output >= CT_CLIP_MAX) return -1;
                output[n_output++] = ib;
            }
            ia = ib;
            a_inside = b_inside;
        }
        if (n_output < 3) {
            *cur_out = output;
            *ncur_out = 0;  // area 0
            return nn;
        }
        r = s;
        ir = i;
    }
    *cur_out = output;
    *ncur_out = n_output;
    return nn;
}

// Gradient of the area of intersection of every pair (ia[t], ib[t]) with
// upstream gradient g[t]; accumulated into gva (subject mesh) and gvb
// (clipper / tree mesh).
__global__ void k_clip_area_grad(const double* __restrict__ va, const int64_t* __restrict__ fa, int Ka,
                                 const double* __restrict__ vb, const int64_t* __restrict__ fb, int Kb,
                                 const int64_t* __restrict__ ia, const int64_t* __restrict__ ib, int64_t n,
                                 const double* __restrict__ g, double* __restrict__ gva, double* __restrict__ gvb,
                                 unsigned int* __restrict__ err) {
    int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double G = g[t];
    if (G == 0.0) return;
    dpt a[CT_MAX_N_VERTEX], b[CT_MAX_N_VERTEX];
    const int64_t* face_a = fa + ia[t] * Ka;
    const int64_t* face_b = fb + ib[t] * Kb;
    int la = gather_polygon(va, face_a, Ka, a);
    int lb = gather_polygon(vb, face_b, Kb, b);
    if (la < 1 || lb < 1) return;
    Clip C;
    short* cur;
    int m;
    int nn = clip_taped(C, a, la, b, lb, &cur, &m);
    if (nn < 0) {
        set_error(err, CT_DEVERR_CLIP);
        return;
    }
    if (m < 3) return;  // area 0: zero gradient
    dpt adj[TAPE_MAX];
    dpt cadj[CT_MAX_N_VERTEX];
    for (int k = 0; k < nn; k++) adj[k] = mkp(0.0, 0.0);
    for (int k = 0; k < lb; k++) cadj[k] = mkp(0.0, 0.0);
    // area = 0.5 * sum_i |cross(U_i, V_i)|: U_2 = p1 - p0, U_i = p0 - p_{i-1}, V_i = p0 - p_i
    const short n0 = cur[0];
    const dpt p0 = C.P[n0];
    for (int i = 2; i < m; i++) {
        const short nu = (i == 2) ? cur[1] : cur[i - 1];
        const short nv = cur[i];
        dpt U = (i == 2) ? vsub(C.P[nu], p0) : vsub(p0, C.P[nu]);
        dpt V = vsub(p0, C.P[nv]);
        double sg = 0.5 * G * sgn(crossp(U, V));
        if (sg == 0.0) continue;
        double ux = sg * V.y, uy = -sg * V.x;   // d/dU
        double vx = -sg * U.y, vy = sg * U.x;   // d/dV
        if (i == 2) {
            acc(&adj[nu], ux, uy);
            acc(&adj[n0], -ux, -uy);
        } else {
            acc(&adj[n0], ux, uy);
            acc(&adj[nu], -ux, -uy);
        }
        acc(&adj[n0], vx, vy);
        acc(&adj[nv], -vx, -vy);
    }
    // intersection nodes, newest first: p = A + t V, t = (N.W) / (N.V),
    // V = B - A, W = R - A, N = perp(U), U = S - R
    for (int k = nn - 1; k >= la; k--) {
        const dpt gk = adj[k];
        if (gk.x == 0.0 && gk.y == 0.0) continue;
        const int ka = C.pa[k], kb = C.pb[k], kr = C.pr[k], ks = C.ps[k];
        const dpt A = C.P[ka], B = C.P[kb], R = b[kr], S = b[ks];
        const dpt U = vsub(S, R), N = mkp(-U.y, U.x), V = vsub(B, A), W = vsub(R, A);
        const double nw = dotp(N, W), nv = dotp(N, V);
        const double tt = nw / nv;
        const double lam = dotp(gk, V) / nv;
        acc(&adj[ka], gk.x * (1.0 - tt), gk.y * (1.0 - tt));
        acc(&adj[kb], gk.x * tt, gk.y * tt);
        // lam * N.dW  (W = R - A) and -lam*t * N.dV  (V = B - A)
        acc(&cadj[kr], lam * N.x, lam * N.y);
        acc(&adj[ka], -lam * N.x + lam * tt * N.x, -lam * N.y + lam * tt * N.y);
        acc(&adj[kb], -lam * tt * N.x, -lam * tt * N.y);
        // lam * dN.W - lam*t * dN.V, dN.X = dU . (X.y, -X.x), U = S - R
        double ux = lam * W.y - lam * tt * V.y, uy = -lam * W.x + lam * tt * V.x;
        acc(&cadj[ks], ux, uy);
        acc(&cadj[kr], -ux, -uy);
    }
    for (int k = 0; k < la; k++) {
        int64_t vi = face_a[k];
        if (adj[k].x != 0.0) atomicAdd(&gva[2 * vi], adj[k].x);
        if (adj[k].y != 0.0) atomicAdd(&gva[2 * vi + 1], adj[k].y);
    }
    for (int k = 0; k < lb; k++) {
        int64_t vi = face_b[k];
        if (cadj[k].x != 0.0) atomicAdd(&gvb[2 * vi], cadj[k].x);
        if (cadj[k].y != 0.0) atomicAdd(&gvb[2 * vi + 1], cadj[k].y);
    }
}

// cross(X, Y) with adjoint d: X += d (Y.y, -Y.x), Y += d (-X.y, X.x)
__device__ __forceinline__ void cross_back(dpt X, dpt Y, double d, dpt* gX, dpt* gY) {
    acc(gX, d * Y.y, -d * Y.x);
    acc(gY, -d * X.y, d * X.x);
}

// Gradient of the barycentric weights (n x KW, upstream gw) with respect to
// the tree vertices (accumulated into gv) and the points (written to gp).
__global__ void k_barycentric_grad(const double2* __restrict__ pts, const int64_t* __restrict__ fidx, int64_t n,
                                   const double* __restrict__ v, const int64_t* __restrict__ faces, int K, int KW,
                                   double tol, const double* __restrict__ gw, double* __restrict__ gv,
                                   double* __restrict__ gp) {
    int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    dpt gpt = mkp(0.0, 0.0);
    const int64_t f = fidx[i];
    if (f != -1) {
        const double2 pp = pts[i];
        const dpt p = mkp(pp.x, pp.y);
        const int64_t* face = faces + f * K;
        const double* G = gw + i * KW;
        dpt poly[CT_MAX_N_VERTEX], gpoly[CT_MAX_N_VERTEX];
        int len;
        if (K > 3) {
            len = gather_polygon(v, face, K, poly);
        } else {
            len = 3;
            for (int k = 0; k < 3; k++) poly[k] = mkp(v[2 * face[k]], v[2 * face[k] + 1]);
        }
        for (int k = 0; k < len; k++) gpoly[k] = mkp(0.0, 0.0);
        if (K <= 3) {
            // barycentric_triangle.py:28-43
            const dpt A0 = poly[0], B0 = poly[1], C0 = poly[2];
            const dpt ab = vsub(B0, A0), ac = vsub(C0, A0), ap = vsub(p, A0);
            const double xa = crossp(ab, ap), xc = crossp(ac, ap), xA = crossp(ab, ac);
            const double Aa = fabs(xa), Ac = fabs(xc), A = fabs(xA);
            const double inv = 1.0 / A;
            const double gW = G[2] - G[0], gV = G[1] - G[0];
            const double g_inv = gW * Aa + gV * Ac;
            const double dxa = gW * inv * sgn(xa), dxc = gV * inv * sgn(xc), dxA = -g_inv * inv * inv * sgn(xA);
            dpt gab = mkp(0, 0), gac = mkp(0, 0), gap = mkp(0, 0);
            cross_back(ab, ap, dxa, &gab, &gap);
            cross_back(ac, ap, dxc, &gac, &gap);
            cross_back(ab, ac, dxA, &gab, &gac);
            acc(&gpoly[1], gab.x, gab.y);
            acc(&gpoly[2], gac.x, gac.y);
            acc(&gpoly[0], -gab.x - gac.x - gap.x, -gab.y - gac.y - gap.y);
            gpt = gap;
        } else {
            // barycentric_wachspress.py:26-85; E_k = cross(v_{k+1} - v_k, p - v_k)
            const int nv = len;
            int edge = -1;  // first edge (in the upstream order) within the tolerance
            {
                dpt U = vsub(poly[0], poly[nv - 1]);
                if (within_perp(fabs(crossp(U, vsub(p, poly[nv - 1]))), U, tol)) edge = nv - 1;
                for (int k = 0; k < nv && edge < 0; k++) {
                    dpt Uk = vsub(poly[(k + 1) % nv], poly[k]);
                    if (within_perp(fabs(crossp(Uk, vsub(p, poly[k]))), Uk, tol)) edge = k;
                }
            }
            if (edge >= 0) {
                // interp_edge_case: w = |p - a| / |U|, weights (1 - w, w) at (edge, edge + 1)
                const int i0 = edge, j0 = (edge + 1) % nv;
                const dpt a = poly[i0];
                const dpt U = vsub(poly[j0], a), V = vsub(p, a);
                const double lv = sqrt(dotp(V, V)), lu = sqrt(dotp(U, U));
                const double w = lv / lu;
                const double gw_ = G[j0] - G[i0];
                dpt gV = mkp(0, 0), gU = mkp(0, 0);
                if (lv > 0.0) gV = mkp(gw_ * V.x / (lv * lu), gw_ * V.y / (lv * lu));
                gU = mkp(-gw_ * w * U.x / (lu * lu), -gw_ * w * U.y / (lu * lu));
                gpt = gV;
                acc(&gpoly[i0], -gV.x - gU.x, -gV.y - gU.y);
                acc(&gpoly[j0], gU.x, gU.y);
            } else {
                double E[CT_MAX_N_VERTEX], Cc[CT_MAX_N_VERTEX], w[CT_MAX_N_VERTEX];
                for (int k = 0; k < nv; k++) {
                    const int k1 = (k + 1) % nv, km = (k + nv - 1) % nv;
                    E[k] = crossp(vsub(poly[k1], poly[k]), vsub(p, poly[k]));
                    Cc[k] = crossp(vsub(poly[k], poly[km]), vsub(poly[k1], poly[km]));
                }
                double S = 0.0;
                for (int k = 0; k < nv; k++) {
                    const int km = (k + nv - 1) % nv;
                    w[k] = 2.0 * fabs(Cc[k]) / (fabs(E[km]) * fabs(E[k]));
                    S += w[k];
                }
                double dot = 0.0;
                for (int k = 0; k < nv; k++) dot += G[k] * (w[k] / S);
                double gE[CT_MAX_N_VERTEX];
                for (int k = 0; k < nv; k++) gE[k] = 0.0;
                for (int k = 0; k < nv; k++) {
                    const int km = (k + nv - 1) % nv, k1 = (k + 1) % nv;
                    const double gwk = (G[k] - dot) / S;
                    const double dC = gwk * 2.0 / (fabs(E[km]) * fabs(E[k])) * sgn(Cc[k]);
                    gE[km] += -gwk * w[k] / fabs(E[km]);
                    gE[k] += -gwk * w[k] / fabs(E[k]);
                    dpt X = vsub(poly[k], poly[km]), Y = vsub(poly[k1], poly[km]);
                    dpt gX = mkp(0, 0), gY = mkp(0, 0);
                    cross_back(X, Y, dC, &gX, &gY);
                    acc(&gpoly[k], gX.x, gX.y);
                    acc(&gpoly[k1], gY.x, gY.y);
                    acc(&gpoly[km], -gX.x - gY.x, -gX.y - gY.y);
                }
                for (int k = 0; k < nv; k++) {
                    const int k1 = (k + 1) % nv;
                    const double dE = gE[k] * sgn(E[k]);
                    dpt D = vsub(poly[k1], poly[k]), Q = vsub(p, poly[k]);
                    dpt gD = mkp(0, 0), gQ = mkp(0, 0);
                    cross_back(D, Q, dE, &gD, &gQ);
                    acc(&gpoly[k1], gD.x, gD.y);
                    acc(&gpoly[k], -gD.x - gQ.x, -gD.y - gQ.y);
                    acc(&gpt, gQ.x, gQ.y);
                }
            }
        }
        for (int k = 0; k < len; k++) {
            const int64_t vi = face[k];
            if (gpoly[k].x != 0.0) atomicAdd(&gv[2 * vi], gpoly[k].x);
            if (gpoly[k].y != 0.0) atomicAdd(&gv[2 * vi + 1], gpoly[k].y);
        }
    }
    if (gp) {
        gp[2 * i] = gpt.x;
        gp[2 * i + 1] = gpt.y;
    }
}

}  // namespace cta

using namespace cta;

extern "C" {

int ct_area_of_intersection_grad(const double* va, const int64_t* fa, int32_t Ka, const double* vb, const int64_t* fb,
                                 int32_t Kb, const int64_t* ia, const int64_t* ib, int64_t n, const double* grad_area,
                                 double* grad_va, double* grad_vb, unsigned int* error_word, void* stream) {
    if (n < 0 || Ka < 1 || Kb < 1 || Ka > CT_MAX_N_VERTEX || Kb > CT_MAX_N_VERTEX)
        return ct_fail(CT_ERR_ARG, "bad sizes");
    if (n == 0) return CT_OK;
    if (!va || !fa || !vb || !fb || !ia || !ib || !grad_area || !grad_va || !grad_vb)
        return ct_fail(CT_ERR_ARG, "null argument");
    unsigned grid = (unsigned)((n + 127) / 128);
    k_clip_area_grad<<<grid, 128, 0, (cudaStream_t)stream>>>(va, fa, Ka, vb, fb, Kb, ia, ib, n, grad_area, grad_va,
                                                             grad_vb, error_word);
    CT_CHECK_LAUNCH("area_of_intersection_grad");
    return CT_OK;
}

int ct_barycentric_weights_grad(const double* points, const int64_t* face_index, int64_t n, const double* vertices,
                                const int64_t* faces, int32_t K, int32_t KW, double tolerance,
                                const double* grad_weights, double* grad_vertices, double* grad_points, void* stream) {
    if (n < 0 || K < 3 || K > CT_MAX_N_VERTEX || KW < K) return ct_fail(CT_ERR_ARG, "bad sizes");
    if (n == 0) return CT_OK;
    if (!points || !face_index || !vertices || !faces || !grad_weights || !grad_vertices)
        return ct_fail(CT_ERR_ARG, "null argument");
    unsigned grid = (unsigned)((n + 127) / 128);
    k_barycentric_grad<<<grid, 128, 0, (cudaStream_t)stream>>>((const double2*)points, face_index, n, vertices, faces,
                                                               K, KW, tolerance, grad_weights, grad_vertices,
                                                               grad_points);
    CT_CHECK_LAUNCH("barycentric_weights_grad");
    return CT_OK;
}

}  // extern "C"
