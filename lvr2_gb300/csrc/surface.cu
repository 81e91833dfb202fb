// surface.cu -- fused kNN + plane fit + flip (AdaptiveKSearchSurface
// calculateSurfaceNormals), normal interpolation, kNN rows and
// getInterpolatedNormal, all on the warp-cooperative LBVH traversal.
#include <algorithm>
#include <atomic>
#include <cstring>
#include <functional>
#include <random>
#include <stdexcept>
#include <unordered_set>
#include <vector>

#include "primitives.cuh"
#include "surface.h"
#include "wide.cuh"

namespace lvrgb {

namespace {

__device__ __forceinline__ void kahan_add(float& s, float& c, float v) {
    float y = __fsub_rn(v, c);
    float t = __fadd_rn(s, y);
    c = __fsub_rn(__fsub_rn(t, s), y);
    s = t;
}

// Eigen-style choice among three eigenvalues (first strictly smallest wins,
// then the second, else the third), as in calcPlaneIPCAExact.
__device__ __forceinline__ int pick_smallest(double e0, double e1, double e2) {
    if (e0 < e1 && e0 < e2) return 0;
    if (e1 < e2) return 1;
    return 2;
}

// Cyclic Jacobi eigen-decomposition in double; smallest eigenvector.  The
// rare fallback of the FP32 solve: kept out of line.
__device__ __noinline__ void jacobi3_smallest(const double Ain[6], double v_out[3]) {
    double A[3][3] = {{Ain[0], Ain[1], Ain[2]}, {Ain[1], Ain[3], Ain[4]}, {Ain[2], Ain[4], Ain[5]}};
    double V[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    for (int sweep = 0; sweep < 50; sweep++) {
        double off = A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2];
        if (off == 0.0) break;
        for (int p = 0; p < 2; p++)
            for (int q = p + 1; q < 3; q++) {
                if (A[p][q] == 0.0) continue;
                double theta = (A[q][q] - A[p][p]) / (2.0 * A[p][q]);
                double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 3; k++) {
                    double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 3; k++) {
                    double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 3; k++) {
                    double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
    }
    int m = pick_smallest(A[0][0], A[1][1], A[2][2]);
    double n = sqrt(V[0][m] * V[0][m] + V[1][m] * V[1][m] + V[2][m] * V[2][m]);
    for (int k = 0; k < 3; k++) v_out[k] = V[k][m] / n;
}

// Smallest eigenvector of a symmetric 3x3 matrix (a00 a01 a02 a11 a12 a22)
// in FP32 by the closed-form trigonometric eigenvalues (Smith 1961) and a
// cross product of two rows of (A - lambda I).  w = 0 when the result is not
// trustworthy in FP32 (relative eigengap below gap_thr or nearly parallel
// rows); the caller then solves in FP64.  Out of line: with its trigonometric
// functions it would otherwise dominate the code size of the kernels that
// inline it.
__device__ __noinline__ float4 eig_smallest_f32(float a00, float a01, float a02, float a11, float a12, float a22,
                                                float gap_thr) {
    const float p1 = a01 * a01 + a02 * a02 + a12 * a12;
    if (p1 == 0.0f) {
        int m = pick_smallest(a00, a11, a22);
        return make_float4(m == 0, m == 1, m == 2, 1.0f);
    }
    const float q = (a00 + a11 + a22) * (1.0f / 3.0f);
    const float b00 = a00 - q, b11 = a11 - q, b22 = a22 - q;
    const float p2 = b00 * b00 + b11 * b11 + b22 * b22 + 2.0f * p1;
    const float p = sqrtf(p2 * (1.0f / 6.0f));
    if (!(p > 0.0f)) return make_float4(0, 0, 0, 0);
    const float ip = 1.0f / p;
    const float c00 = b00 * ip, c11 = b11 * ip, c22 = b22 * ip;
    const float c01 = a01 * ip, c02 = a02 * ip, c12 = a12 * ip;
    const float det = c00 * (c11 * c22 - c12 * c12) - c01 * (c01 * c22 - c12 * c02) + c02 * (c01 * c12 - c11 * c02);
    const float r = fminf(fmaxf(0.5f * det, -1.0f), 1.0f);
    const float phi = acosf(r) * (1.0f / 3.0f);
    const float l1 = q + 2.0f * p * cosf(phi);
    const float l3 = q + 2.0f * p * cosf(phi + 2.0943951023931953f);
    const float l2 = 3.0f * q - l1 - l3;
    const float scale = fmaxf(fabsf(l1), 1e-30f);
    if ((l2 - l3) < gap_thr * scale) return make_float4(0, 0, 0, 0);
    const float r0[3] = {a00 - l3, a01, a02};
    const float r1[3] = {a01, a11 - l3, a12};
    const float r2[3] = {a02, a12, a22 - l3};
    float x[3][3];
    x[0][0] = r0[1] * r1[2] - r0[2] * r1[1];
    x[0][1] = r0[2] * r1[0] - r0[0] * r1[2];
    x[0][2] = r0[0] * r1[1] - r0[1] * r1[0];
    x[1][0] = r0[1] * r2[2] - r0[2] * r2[1];
    x[1][1] = r0[2] * r2[0] - r0[0] * r2[2];
    x[1][2] = r0[0] * r2[1] - r0[1] * r2[0];
    x[2][0] = r1[1] * r2[2] - r1[2] * r2[1];
    x[2][1] = r1[2] * r2[0] - r1[0] * r2[2];
    x[2][2] = r1[0] * r2[1] - r1[1] * r2[0];
    float best = -1.0f;
    int bi = 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
        float nn = x[i][0] * x[i][0] + x[i][1] * x[i][1] + x[i][2] * x[i][2];
        if (nn > best) { best = nn; bi = i; }
    }
    const float rn = fmaxf(fmaxf(r0[0] * r0[0] + r0[1] * r0[1] + r0[2] * r0[2],
                                 r1[0] * r1[0] + r1[1] * r1[1] + r1[2] * r1[2]),
                           r2[0] * r2[0] + r2[1] * r2[1] + r2[2] * r2[2]);
    if (!(best > 1e-10f * rn * rn)) return make_float4(0, 0, 0, 0);
    const float inv = rsqrtf(best);
    return make_float4(x[bi][0] * inv, x[bi][1] * inv, x[bi][2] * inv, 1.0f);
}

struct NormalsArgs {
    Lbvh T;
    int K;
    int nem;
    int adaptive;
    int last_round;
    int round;  // 1..5
    const uint32_t* list;
    int nq;
    float fx, fy, fz;
    float gap_thr;
    float4* normals;
    int32_t* kused;
    uint8_t* flags;  // per query of the round: 1 = search again with a larger k
    // Squared distance of the k-th neighbour of every point that searches
    // again (by Morton position): written by a round, read by the next one.
    float* kth_d2;
    // Optional per point (Morton position): a flip point of its own when w != 0
    // (the nearest scan pose's point, AdaptiveKSearchSurface.tcc:252-265).
    const float4* flip_target;
    int wide_tile;  // queries per warp tile of the one-warp-per-query kernel (1..32)
    unsigned long long* gheap;
    int* err;
    uint32_t* stats;
    uint32_t* nbr;  // optional: first ki neighbours (Morton positions), column s at nbr[s * n]
    int ki;
    // Segmented (multi-scan) mode: per-bucket scan id and per-scan search
    // root, bucket range and flip point; nq_dev replaces nq when given.
    const SegInfo* segs;
    const uint16_t* bucket_scan;
    const uint32_t* nq_dev;
    // Collapsed rounds (one-warp-per-query kernel only): this launch is the
    // last round's search (K = 32 kn) standing in for rounds round_prefix0 ..
    // 5.  kNN(k) is the first k of kNN(K) in (d2, index) order, so the first
    // kprefix[p] neighbours are exactly the search of round round_prefix0 + p;
    // the first of them whose box test passes is fitted, as the round-by-round
    // sequence would.  nprefix = 0: a plain round.
    int nprefix = 0;
    int kprefix[3] = {0, 0, 0};
    int round_prefix0 = 0;
    // one-warp-per-query launch shape requested by the caller (0: automatic)
    // and its key-buffer size in units of K
    int wide_tile_req = 0;
    int wide_slack = 2;
    // Scale from the previous round's k-th squared distance to a search bound:
    // 2.5 per doubling of k (the squared k-th distance grows by 2 on a surface,
    // 4 along a line; above 2 most searches need no second pass).
    float bound_growth = 2.5f;
    int* tiles = nullptr;  // tile counter of a persistent per-lane launch
};


// BaseVector::normalize with IEEE operations (null vector unchanged).
__device__ __forceinline__ void normalize_ieee(float& x, float& y, float& z) {
    if (!(x == 0.0f && y == 0.0f && z == 0.0f)) {
        float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)), __fmul_rn(z, z)));
        x = __fdiv_rn(x, len);
        y = __fdiv_rn(y, len);
        z = __fdiv_rn(z, len);
    }
}

// First pass over the neighbourhood: bounding box (for the adaptive-k test)
// and the sums each plane fit needs.  Real heap entries occupy [0, cnt).
struct NbrPass {
    float lo[3], hi[3];
    float s[3], c[3];  // compensated sums of p - q (nem 0 and 3)
    float r[6];        // sums of (p - q)(p - q)^T in IEEE order (nem 2)
};

// point_at(s): the s-th neighbour's point, ascending (d2, index) order.
template <int kNem, class PointAt>
__device__ __forceinline__ void neighbour_pass(PointAt point_at, int cnt, float4 q, NbrPass& P) {
#pragma unroll
    for (int a = 0; a < 3; a++) {
        P.lo[a] = FLT_MAX; P.hi[a] = -FLT_MAX; P.s[a] = 0.0f; P.c[a] = 0.0f;
    }
#pragma unroll
    for (int a = 0; a < 6; a++) P.r[a] = 0.0f;
#pragma unroll 4
    for (int s = 0; s < cnt; s++) {
        const float4 p = point_at(s);
        P.lo[0] = fminf(p.x, P.lo[0]); P.lo[1] = fminf(p.y, P.lo[1]); P.lo[2] = fminf(p.z, P.lo[2]);
        P.hi[0] = fmaxf(p.x, P.hi[0]); P.hi[1] = fmaxf(p.y, P.hi[1]); P.hi[2] = fmaxf(p.z, P.hi[2]);
        if (kNem == 4) {
            // the box only (nem 4 sums in FP64 in lbvh_plane_fit)
        } else if (kNem == 2) {
            const float rx = __fsub_rn(p.x, q.x), ry = __fsub_rn(p.y, q.y), rz = __fsub_rn(p.z, q.z);
            P.r[0] = __fadd_rn(P.r[0], __fmul_rn(rx, rx));
            P.r[1] = __fadd_rn(P.r[1], __fmul_rn(rx, ry));
            P.r[2] = __fadd_rn(P.r[2], __fmul_rn(rx, rz));
            P.r[3] = __fadd_rn(P.r[3], __fmul_rn(ry, ry));
            P.r[4] = __fadd_rn(P.r[4], __fmul_rn(ry, rz));
            P.r[5] = __fadd_rn(P.r[5], __fmul_rn(rz, rz));
        } else {
            kahan_add(P.s[0], P.c[0], p.x - q.x);
            kahan_add(P.s[1], P.c[1], p.y - q.y);
            kahan_add(P.s[2], P.c[2], p.z - q.z);
        }
    }
}

// Mean of the neighbourhood relative to q: nem 3 includes q itself
// (calcPlaneIPCAExact starts its incremental mean at the query point).
template <int kNem>
__device__ __forceinline__ void plane_mean(const float s[3], int cnt, float mean[3]) {
    const float m = kNem == 3 ? float(cnt + 1) : float(cnt > 0 ? cnt : 1);
    mean[0] = s[0] / m;
    mean[1] = s[1] / m;
    mean[2] = s[2] / m;
}

// Plane normal from the neighbourhood sums.
//   nem 3: S = covariance sums about the centroid, q included (xx xy xz yy yz zz)
//   nem 0: S = sums about the centroid (xx xz zz xy zy); mean relative to q
//   nem 2: r = sums of (p - q)(p - q)^T in IEEE order
template <int kNem>
__device__ __forceinline__ void solve_plane(float gap_thr, float4 q, const float mean[3], const float S[6],
                                            const float r[6], float n[3], bool& fp64) {
    fp64 = false;
    if (kNem == 3) {
        const float4 v = eig_smallest_f32(S[0], S[1], S[2], S[3], S[4], S[5], gap_thr);
        if (v.w != 0.0f) {
            n[0] = v.x; n[1] = v.y; n[2] = v.z;
        } else {
            double D[6], w[3];
            for (int i = 0; i < 6; i++) D[i] = double(S[i]);
            jacobi3_smallest(D, w);
            n[0] = float(w[0]); n[1] = float(w[1]); n[2] = float(w[2]);
            fp64 = true;
        }
    } else if (kNem == 2) {
        // calcPlaneIterative: the largest of the three cofactor determinants
        // of the sums of (p - q)(p - q)^T.
        const float xx = r[0], xy = r[1], xz = r[2], yy = r[3], yz = r[4], zz = r[5];
        const float det_x = __fsub_rn(__fmul_rn(yy, zz), __fmul_rn(yz, yz));
        const float det_y = __fsub_rn(__fmul_rn(xx, zz), __fmul_rn(xz, xz));
        const float det_z = __fsub_rn(__fmul_rn(xx, yy), __fmul_rn(xy, xy));
        float dx, dy, dz;
        if (det_x >= det_y && det_x >= det_z) {
            dx = 1.0f;
            dy = __fdiv_rn(__fsub_rn(__fmul_rn(xz, yz), __fmul_rn(xy, zz)), det_x);
            dz = __fdiv_rn(__fsub_rn(__fmul_rn(xy, yz), __fmul_rn(xz, yy)), det_x);
        } else if (det_y >= det_x && det_y >= det_z) {
            dx = __fdiv_rn(__fsub_rn(__fmul_rn(yz, xz), __fmul_rn(xy, zz)), det_y);
            dy = 1.0f;
            dz = __fdiv_rn(__fsub_rn(__fmul_rn(xy, xz), __fmul_rn(yz, xx)), det_y);
        } else {
            dx = __fdiv_rn(__fsub_rn(__fmul_rn(yz, xy), __fmul_rn(xz, yy)), det_z);
            dy = __fdiv_rn(__fsub_rn(__fmul_rn(xz, xy), __fmul_rn(yz, xx)), det_z);
            dz = 1.0f;
        }
        const float invnorm = __fdiv_rn(1.0f, __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                                  __fmul_rn(dz, dz))));
        n[0] = __fmul_rn(dx, invnorm);
        n[1] = __fmul_rn(dy, invnorm);
        n[2] = __fmul_rn(dz, invnorm);
    } else {
        // calcPlane (nem 0): least-squares y = C0 + C1 x + C2 z over the
        // neighbours; centred FP32 sums relative to q, 2x2 solve in FP64,
        // then the reference's two in-plane vectors at +100 offsets.
        const float mx = mean[0], my = mean[1], mz = mean[2];
        const double sxx = S[0], sxz = S[1], szz = S[2], sxy = S[3], szy = S[4];
        const double det = sxx * szz - sxz * sxz;
        double c1 = 0, c2 = 0;
        if (det != 0) {
            c1 = (sxy * szz - szy * sxz) / det;
            c2 = (szy * sxx - sxy * sxz) / det;
        }
        const double c0 = (double(q.y) + double(my)) - c1 * (double(q.x) + double(mx)) - c2 * (double(q.z) + double(mz));
        const float C0 = float(c0), C1 = float(c1), C2 = float(c2);
        const float eps = 100.0f;
        const float z1 = __fadd_rn(__fadd_rn(C0, __fmul_rn(C1, __fadd_rn(q.x, eps))), __fmul_rn(C2, q.z));
        const float z2 = __fadd_rn(__fadd_rn(C0, __fmul_rn(C1, q.x)), __fmul_rn(C2, __fadd_rn(q.z, eps)));
        const float d1x = __fsub_rn(__fadd_rn(q.x, eps), q.x), d1y = __fsub_rn(z1, q.y), d1z = 0.0f;
        const float d2x = 0.0f, d2y = __fsub_rn(z2, q.y), d2z = __fsub_rn(__fadd_rn(q.z, eps), q.z);
        float nx = __fsub_rn(__fmul_rn(d1y, d2z), __fmul_rn(d1z, d2y));
        float ny = __fsub_rn(__fmul_rn(d1z, d2x), __fmul_rn(d1x, d2z));
        float nz = __fsub_rn(__fmul_rn(d1x, d2y), __fmul_rn(d1y, d2x));
        normalize_ieee(nx, ny, nz);
        n[0] = nx; n[1] = ny; n[2] = nz;
    }
}

// Second pass over a lane's heap: the centred sums of nem 3 / nem 0.
template <int kNem, class PointAt>
__device__ __forceinline__ void centred_sums(PointAt point_at, int cnt, float4 q, const float mean[3], float S[6]) {
    const float mx = mean[0], my = mean[1], mz = mean[2];
    float C[6] = {0, 0, 0, 0, 0, 0};
    if (kNem == 3) {
        // the query point itself, then the neighbours
        S[0] = mx * mx; S[1] = mx * my; S[2] = mx * mz; S[3] = my * my; S[4] = my * mz; S[5] = mz * mz;
    } else {
        for (int i = 0; i < 6; i++) S[i] = 0.0f;
    }
#pragma unroll 4
    for (int s = 0; s < cnt; s++) {
        const float4 p = point_at(s);
        const float ex = (p.x - q.x) - mx, ey = (p.y - q.y) - my, ez = (p.z - q.z) - mz;
        if (kNem == 3) {
            kahan_add(S[0], C[0], ex * ex);
            kahan_add(S[1], C[1], ex * ey);
            kahan_add(S[2], C[2], ex * ez);
            kahan_add(S[3], C[3], ey * ey);
            kahan_add(S[4], C[4], ey * ez);
            kahan_add(S[5], C[5], ez * ez);
        } else {
            kahan_add(S[0], C[0], ex * ex);
            kahan_add(S[1], C[1], ex * ez);
            kahan_add(S[2], C[2], ez * ez);
            kahan_add(S[3], C[3], ex * ey);
            kahan_add(S[4], C[4], ez * ey);
        }
    }
}

template <int kNem, class PointAt>
__device__ __forceinline__ void fit_plane(const NormalsArgs& A, PointAt point_at, int cnt, float4 q, const NbrPass& P,
                                          float n[3], bool& fp64) {
    float mean[3] = {0, 0, 0}, S[6] = {0, 0, 0, 0, 0, 0};
    if (kNem != 2) {
        plane_mean<kNem>(P.s, cnt, mean);
        centred_sums<kNem>(point_at, cnt, q, mean, S);
    }
    solve_plane<kNem>(A.gap_thr, q, mean, S, P.r, n, fp64);
}

// nem 4: the plane fit of lvr2's LBVH comparator (LBVHIndex::knn_normals,
// src/liblvr2/reconstruction/cuda/lbvh/knn_normals_kernel.cu:54-206), used by
// CudaKSearchSurface (--pcm LBVH_CUDA): in FP64, the centroid and covariance
// of neighbours 1..n-1 (slot 0 is the query itself), each term divided by
// n - 1 before it is added; the det^2-weighted sum of the three cofactor axes
// (sign-aligned with the running sum), normalised; flipped toward the flip
// point; a NaN or infinite flip product, or fewer than 3 neighbours, gives the
// zero normal.  Every operation is rounded on its own (no contraction), in
// the reference's order.  Neighbours in ascending (d2, index) order.
// point(s): the s-th neighbour (float4; s in 1..cnt-1).
template <class Point>
__device__ __forceinline__ void lbvh_plane_fit(Point point, int cnt, float qx, float qy, float qz, float fx, float fy,
                                               float fz, float n[3]) {
    n[0] = n[1] = n[2] = 0.0f;
    if (cnt < 3) return;
    const double nf = __dsub_rn(double(cnt), 1.0);
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int s = 1; s < cnt; s++) {
        const float4 p = point(s);
        sx = __dadd_rn(sx, __ddiv_rn(double(p.x), nf));
        sy = __dadd_rn(sy, __ddiv_rn(double(p.y), nf));
        sz = __dadd_rn(sz, __ddiv_rn(double(p.z), nf));
    }
    double xx = 0.0, xy = 0.0, xz = 0.0, yy = 0.0, yz = 0.0, zz = 0.0;
    for (int s = 1; s < cnt; s++) {
        const float4 p = point(s);
        const double rx = __dsub_rn(double(p.x), sx), ry = __dsub_rn(double(p.y), sy), rz = __dsub_rn(double(p.z), sz);
        xx = __dadd_rn(xx, __ddiv_rn(__dmul_rn(rx, rx), nf));
        xy = __dadd_rn(xy, __ddiv_rn(__dmul_rn(rx, ry), nf));
        xz = __dadd_rn(xz, __ddiv_rn(__dmul_rn(rx, rz), nf));
        yy = __dadd_rn(yy, __ddiv_rn(__dmul_rn(ry, ry), nf));
        yz = __dadd_rn(yz, __ddiv_rn(__dmul_rn(ry, rz), nf));
        zz = __dadd_rn(zz, __ddiv_rn(__dmul_rn(rz, rz), nf));
    }
    double wx = 0.0, wy = 0.0, wz = 0.0;
    auto add_axis = [&](double ax, double ay, double az, double det) {
        double w = __dmul_rn(det, det);
        const double dot = __dadd_rn(__dadd_rn(__dmul_rn(wx, ax), __dmul_rn(wy, ay)), __dmul_rn(wz, az));
        if (dot < 0.0) w = -w;
        wx = __dadd_rn(wx, __dmul_rn(ax, w));
        wy = __dadd_rn(wy, __dmul_rn(ay, w));
        wz = __dadd_rn(wz, __dmul_rn(az, w));
    };
    const double det_x = __dsub_rn(__dmul_rn(yy, zz), __dmul_rn(yz, yz));
    add_axis(det_x, __dsub_rn(__dmul_rn(xz, yz), __dmul_rn(xy, zz)), __dsub_rn(__dmul_rn(xy, yz), __dmul_rn(xz, yy)),
             det_x);
    const double det_y = __dsub_rn(__dmul_rn(xx, zz), __dmul_rn(xz, xz));
    add_axis(__dsub_rn(__dmul_rn(xz, yz), __dmul_rn(xy, zz)), det_y, __dsub_rn(__dmul_rn(xy, xz), __dmul_rn(yz, xx)),
             det_y);
    const double det_z = __dsub_rn(__dmul_rn(xx, yy), __dmul_rn(xy, xy));
    add_axis(__dsub_rn(__dmul_rn(xy, yz), __dmul_rn(xz, yy)), __dsub_rn(__dmul_rn(xy, xz), __dmul_rn(yz, xx)), det_z,
             det_z);
    const double mag = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(wx, wx), __dmul_rn(wy, wy)), __dmul_rn(wz, wz)));
    wx = __ddiv_rn(wx, mag);
    wy = __ddiv_rn(wy, mag);
    wz = __ddiv_rn(wz, mag);
    const double dx = __dsub_rn(double(fx), double(qx)), dy = __dsub_rn(double(fy), double(qy)),
                 dz = __dsub_rn(double(fz), double(qz));
    const double scalar = __dadd_rn(__dadd_rn(__dmul_rn(dx, wx), __dmul_rn(dy, wy)), __dmul_rn(dz, wz));
    if (!(scalar <= 0.0 || scalar >= 0.0) || isinf(scalar)) {
        wx = 0.0; wy = 0.0; wz = 0.0;
    }
    if (scalar < 0.0) {
        wx = -wx; wy = -wy; wz = -wz;
    }
    n[0] = float(wx);
    n[1] = float(wy);
    n[2] = float(wz);
}

// LBVHIndex::calculate_normals (src/liblvr2/reconstruction/cuda/LBVHIndex.cu:586-642,
// lbvh/normals_kernel.cu:11-180): the same fit from given neighbour lists,
// one thread per query.  idx rows of k input indices (checked < n by the
// caller), cnt[i] <= k of them used; the query position comes from queries.
__global__ void list_normals_kernel(Lbvh T, const float* __restrict__ queries, int nq, int k,
                                    const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ idx, float fx,
                                    float fy, float fz, float* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const uint32_t* row = idx + size_t(i) * size_t(k);
    float n[3];
    lbvh_plane_fit([&](int s) { return __ldg(T.pts + __ldg(T.inv + row[s])); }, int(cnt[i]),
                   queries[3 * size_t(i)], queries[3 * size_t(i) + 1], queries[3 * size_t(i) + 2], fx, fy, fz, n);
    out[3 * size_t(i)] = n[0];
    out[3 * size_t(i) + 1] = n[1];
    out[3 * size_t(i) + 2] = n[2];
}

// kMinBlocks: resident blocks the register budget must allow.  With heaps of
// k >= 36 the shared memory allows at most five blocks, and at that bound
// (up to 102 registers) the kernel runs without spills; smaller heaps leave
// room for more blocks: six (up to 85 registers) at k = 20 was 2.7% faster
// on a 76M-point scan project than five without spills.
template <int kNem, int kMinBlocks, class Heap = LaneHeap>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, kMinBlocks) normals_kernel(NormalsArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    const int nq = A.nq_dev ? int(*A.nq_dev) : A.nq;
    TravStats st;
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        bool active = qi < nq;
        const int pos = active ? (A.list ? int(A.list[qi]) : qi) : 0;
        const float4 q = __ldg(A.T.pts + pos);
        // padding after each scan of a segmented tree is not a query
        if (A.segs && __float_as_uint(q.w) == 0xffffffffu) active = false;
        Heap heap;
        heap.init(ctx.heap, A.K);
        float fx = A.fx, fy = A.fy, fz = A.fz;
        if (A.segs) {
            // One search per scan present in the warp; each lane searches its own scan's tree.
            const int sc = active ? int(A.bucket_scan[pos / A.T.bucket]) : -1;
            unsigned remaining = __ballot_sync(kFull, active);
            while (remaining) {
                const int leader = __ffs(remaining) - 1;
                const int s = __shfl_sync(kFull, sc, leader);
                const unsigned grp = __ballot_sync(kFull, active && sc == s);
                remaining &= ~grp;
                const SegInfo g = A.segs[s];
                const int seed = __shfl_sync(kFull, pos, leader) / A.T.bucket;
                knn_traverse(A.T, q.x, q.y, q.z, (grp >> lane) & 1u, heap, ctx.stage, A.err, st, seed, g.root,
                             g.blo, g.bhi);
            }
            if (active) {
                fx = A.segs[sc].fx; fy = A.segs[sc].fy; fz = A.segs[sc].fz;
            }
        } else {
            const int seed = __shfl_sync(kFull, pos, 0) / A.T.bucket;
            knn_traverse(A.T, q.x, q.y, q.z, active, heap, ctx.stage, A.err, st, seed);
        }
        if (A.flip_target && active) {
            const float4 t = __ldg(A.flip_target + pos);
            if (t.w != 0.0f) {
                fx = t.x; fy = t.y; fz = t.z;
            }
        }
        bool retry = false;
        if (active) {
            // Ascending order puts the real entries first (fewer points than K),
            // gives the interpolation its ki nearest in lvr2's order, and makes
            // the sums below independent of the order the search met the
            // neighbours in (any tree over the same points gives the same normal).
            const int cnt = heap.real;
            heap.sort_ascending();
            NbrPass P;
            // The first pass looks each neighbour's Morton position up once and
            // keeps it in the low word of its key (the order is already fixed),
            // so the later passes and the interpolation lists read it directly.
            unsigned long long* hk = heap.h;
            const auto first_point = [&](int s) {
                const unsigned long long k = hk[s * 32];
                const uint32_t at = __ldg(A.T.inv + key_idx(k));
                hk[s * 32] = (k & 0xffffffff00000000ull) | at;
                return __ldg(A.T.pts + at);
            };
            const auto point_at = [&](int s) { return __ldg(A.T.pts + key_idx(hk[s * 32])); };
            neighbour_pass<kNem>(first_point, cnt, q, P);
            bool fit = true;
            if (A.adaptive && !A.last_round) {
                // boundingBoxOK over the neighbourhood (AdaptiveKSearchSurface.tcc:337-350)
                const float dx = __fsub_rn(P.hi[0], P.lo[0]), dy = __fsub_rn(P.hi[1], P.lo[1]),
                            dz = __fsub_rn(P.hi[2], P.lo[2]);
                const float e = 0.05f;
                fit = dx >= __fmul_rn(e, dy) && dx >= __fmul_rn(e, dz) && dy >= __fmul_rn(e, dx) &&
                      dy >= __fmul_rn(e, dz) && dz >= __fmul_rn(e, dx) && dz >= __fmul_rn(e, dy);
            }
            if (fit) {
                float n[3];
                bool fp64 = false;
                if (kNem == 4) {
                    lbvh_plane_fit(point_at, cnt, q.x, q.y, q.z, fx, fy, fz, n);
                } else {
                    fit_plane<kNem>(A, point_at, cnt, q, P, n, fp64);
                    // Flip toward the flip point; Normal::operator-() re-normalises.
                    const float tx = __fsub_rn(fx, q.x), ty = __fsub_rn(fy, q.y), tz = __fsub_rn(fz, q.z);
                    const float dot =
                        __fadd_rn(__fadd_rn(__fmul_rn(n[0], tx), __fmul_rn(n[1], ty)), __fmul_rn(n[2], tz));
                    if (dot < 0.0f) {
                        n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2];
                        normalize_ieee(n[0], n[1], n[2]);
                    }
                }
                A.normals[pos] = make_float4(n[0], n[1], n[2], 0.0f);
                if (A.kused) A.kused[pos] = A.K;
                if (A.nbr) {
                    // kNN(ki) of the interpolation = the first ki of this kNN(K >= ki)
                    for (int j = 0; j < A.ki; j++)
                        A.nbr[size_t(j) * A.T.n + pos] = j < cnt ? key_idx(hk[j * 32]) : 0xffffffffu;
                }
                if (fp64) atomicAdd(A.stats + 5, 1u);
            } else {
                retry = true;
                if (A.kth_d2) A.kth_d2[pos] = cnt == A.K ? heap.tau() : __int_as_float(0x7f800000);
            }
        }
        const unsigned fitted = __ballot_sync(kFull, active && !retry);
        if (lane == 0 && fitted) atomicAdd(A.stats + (A.round - 1), uint32_t(__popc(fitted)));
        if (qi < nq) A.flags[qi] = retry ? 1 : 0;
    }
    unsigned pushes = st.pushes;
    for (int o = 16; o > 0; o >>= 1) pushes += __shfl_xor_sync(kFull, pushes, o);
    if (lane == 0 && st.nodes) {
        atomicAdd(A.stats + 8, st.buckets);
        atomicAdd(A.stats + 9, st.nodes);
        atomicAdd(A.stats + 10, pushes);
        atomicAdd(A.stats + 11, st.chunks);
        atomicAdd(A.stats + 12, st.rounds);
    }
}

// normals_kernel for K > kSmemHeapMax: one warp per query (wide.cuh), the
// neighbourhood sums reduced across the warp.  The neighbour set, the box
// test and therefore the round in which a point is fitted are the same as in
// the per-lane kernel.  With collapsed rounds (A.nprefix > 0) the launch is
// the last round's search, and the rounds it stands in for are tested on the
// prefixes of its kNN; a prefix of at most kSmemHeapMax keys is fitted with
// the per-lane kernel's arithmetic, a longer one with this kernel's, as the
// rounds would have been run one by one.
// x * 2^e, exact unless the result leaves the normal range.
__device__ __forceinline__ float mul_pow2(float x, int e) {
    while (e > 126) {
        x = __fmul_rn(x, __int_as_float(253 << 23));  // 2^126
        e -= 126;
    }
    while (e < -126) {
        x = __fmul_rn(x, __int_as_float(1 << 23));  // 2^-126
        e += 126;
    }
    return __fmul_rn(x, __int_as_float((e + 127) << 23));
}

// E with |p - q| < 2^E for every point p of the box [lo, hi].
__device__ __forceinline__ int box_exponent(const float lo[3], const float hi[3], float4 q) {
    const float m = fmaxf(fmaxf(fmaxf(fabsf(__fsub_rn(lo[0], q.x)), fabsf(__fsub_rn(hi[0], q.x))),
                                fmaxf(fabsf(__fsub_rn(lo[1], q.y)), fabsf(__fsub_rn(hi[1], q.y)))),
                          fmaxf(fabsf(__fsub_rn(lo[2], q.z)), fabsf(__fsub_rn(hi[2], q.z))));
    if (!(m > 0.0f) || !(m <= FLT_MAX)) return 0;
    const unsigned b = __float_as_uint(m);
    const int biased = int(b >> 23);
    if (biased == 0) return 32 - __clz(int(b)) - 149;  // subnormal: m = b * 2^-149
    return biased - 126;                               // m = 1.f * 2^(biased - 127)
}

// 64-bit fixed point with 40 fractional bits: terms below 4 in magnitude and
// up to 2^20 of them stay below 2^62.
__device__ __forceinline__ long long to_fixed(float v) {
    return __float2ll_rn(__fmul_rn(v, 1099511627776.0f));  // 2^40
}
__device__ __forceinline__ float from_fixed(long long v) { return float(double(v) * (1.0 / 1099511627776.0)); }

__device__ __forceinline__ long long warp_sum_ll(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
    return v;
}

constexpr int kWideWarps = 8;  // warps per block
constexpr int kWideTileMax = 32;  // queries per warp tile (consecutive queries chain their bounds)

// kPrefix: compiled with the collapsed-round code (A.nprefix read); without
// it the kernel keeps the registers of a plain round.
template <int kNem, bool kPrefix>
__global__ void __launch_bounds__(kWideWarps * 32, 4) normals_wide_kernel(NormalsArgs A) {
    const int nprefix = kPrefix ? A.nprefix : 0;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WideState W;
    W.K = A.K;
    W.cap = wide_capacity(A.K, A.wide_slack);
    W.hist = reinterpret_cast<uint32_t*>(smem) + wib * 256;
    W.keys = A.gheap ? A.gheap + (size_t(blockIdx.x) * kWideWarps + wib) * size_t(W.cap)
                     : reinterpret_cast<unsigned long long*>(smem + kWideWarps * 1024) + size_t(wib) * W.cap;
    const int nq = A.nq_dev ? int(*A.nq_dev) : A.nq;
    const int B = A.T.bucket;
    TravStats st;
    const int TQ = A.wide_tile;
    for (int tile = first_tile<kWideWarps>(A.tiles); tile * TQ < nq; tile = next_tile<kWideWarps>(A.tiles, tile)) {
        unsigned fitted = 0, retry = 0;
        const int nt = min(TQ, nq - tile * TQ);
        // the previous query of this tile: position, k-th squared distance, scan
        float cx = 0, cy = 0, cz = 0, ctau = __int_as_float(0x7f800000);
        int cscan = -1;
        for (int j = 0; j < nt; j++) {
            const int qi = tile * TQ + j;
            const int pos = A.list ? int(__ldg(A.list + qi)) : qi;
            const float4 q = __ldg(A.T.pts + pos);
            int root = 0, blo = 0, bhi = 0x7fffffff, scan = 0;
            float fx = A.fx, fy = A.fy, fz = A.fz;
            if (A.segs) {
                if (__float_as_uint(q.w) == 0xffffffffu) continue;  // padding after a scan
                scan = A.bucket_scan[pos / B];
                const SegInfo g = A.segs[scan];
                root = g.root; blo = g.blo; bhi = g.bhi;
                fx = g.fx; fy = g.fy; fz = g.fz;
            }
            if (A.flip_target) {
                const float4 t = __ldg(A.flip_target + pos);
                if (t.w != 0.0f) {
                    fx = t.x; fy = t.y; fz = t.z;
                }
            }
            // Search bounds, each exact when at least K points lie within it:
            //  * chain: the previous query's K points lie within
            //    (sqrt(ctau) + |q - q_prev|) of q (triangle inequality; a
            //    relative margin covers the float rounding), so this bound
            //    holds them,
            //  * estimate: the previous round's k-th distance of this point,
            //    scaled for twice the k, which may hold fewer.
            // A search that finds fewer than K points within its bound runs
            // again with the next larger one, the last without a bound.
            const float inf = __int_as_float(0x7f800000);
            float chain = inf;
            if (ctau < FLT_MAX && cscan == scan) {
                const float dx = __fsub_rn(q.x, cx), dy = __fsub_rn(q.y, cy), dz = __fsub_rn(q.z, cz);
                const float delta = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                         __fmul_rn(dz, dz)));
                const float r = __fmul_rn(__fadd_rn(__fsqrt_rn(ctau), delta), 1.0000038f);
                chain = __fmul_rn(__fmul_rn(r, r), 1.0000038f);
            }
            float estimate = inf;
            if (A.round > 1 && A.kth_d2) {
                const float prev = A.kth_d2[pos];
                if (prev < FLT_MAX) estimate = __fmul_rn(prev, A.bound_growth);
            }
            float bound = fminf(chain, estimate);
            for (int attempt = 0; attempt < 3; attempt++) {
                wide_knn(A.T, q.x, q.y, q.z, W, A.err, st, pos / B, root, blo, bhi, bound);
                if (W.cnt >= W.K || !(bound < FLT_MAX)) break;
                bound = (bound < chain && chain < FLT_MAX) ? chain : inf;
                st.retries++;
            }
            st.rounds++;
            const int cnt = W.cnt;
            // the K-th key of this query bounds the next one's search
            ctau = inf;
            if (cnt == W.K) {
                unsigned long long mx = 0;
                for (int i = lane; i < cnt; i += 32) mx = max(mx, W.keys[i]);
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
                ctau = key_d2(mx);
                cx = q.x; cy = q.y; cz = q.z;
                cscan = scan;
            }
            // The neighbourhood that is fitted: with collapsed rounds the first
            // kprefix[p] keys (those at or below their k-th key, use_thr) of
            // the first round whose box test passes, else all cnt keys.
            int use_cnt = cnt, fit_round = A.round, kfit = A.K;
            unsigned long long use_thr = ~0ull;
            float lo[3], hi[3];
            bool fit = false;
            for (int pr = 0; pr <= nprefix && !fit; pr++) {
                const bool full = pr == nprefix;
                const int m = full ? cnt : min(A.kprefix[pr], cnt);
                const unsigned long long thr = (m == cnt || m <= 0) ? ~0ull : warp_select(W.keys, cnt, m, W.hist);
                // neighbourhood box (min / max: exact in any order)
                lo[0] = lo[1] = lo[2] = FLT_MAX;
                hi[0] = hi[1] = hi[2] = -FLT_MAX;
                for (int i = lane; i < cnt; i += 32) {
                    const unsigned long long key = W.keys[i];
                    if (key > thr) continue;
                    const float4 p = neighbour_point(A.T, key);
                    lo[0] = fminf(p.x, lo[0]); lo[1] = fminf(p.y, lo[1]); lo[2] = fminf(p.z, lo[2]);
                    hi[0] = fmaxf(p.x, hi[0]); hi[1] = fmaxf(p.y, hi[1]); hi[2] = fmaxf(p.z, hi[2]);
                }
#pragma unroll
                for (int a = 0; a < 3; a++) {
                    lo[a] = warp_min_f(lo[a]);
                    hi[a] = warp_max_f(hi[a]);
                }
                fit = true;
                if (A.adaptive && !(full && A.last_round)) {
                    // boundingBoxOK over the neighbourhood (AdaptiveKSearchSurface.tcc:337-350)
                    const float dx = __fsub_rn(hi[0], lo[0]), dy = __fsub_rn(hi[1], lo[1]),
                                dz = __fsub_rn(hi[2], lo[2]);
                    const float e = 0.05f;
                    fit = dx >= __fmul_rn(e, dy) && dx >= __fmul_rn(e, dz) && dy >= __fmul_rn(e, dx) &&
                          dy >= __fmul_rn(e, dz) && dz >= __fmul_rn(e, dx) && dz >= __fmul_rn(e, dy);
                }
                if (fit && !full) {
                    use_cnt = m;
                    use_thr = thr;
                    fit_round = A.round_prefix0 + pr;
                    kfit = A.kprefix[pr];
                }
            }
            if (!fit) {
                retry |= 1u << j;
                if (A.kth_d2 && lane == 0) A.kth_d2[pos] = ctau;
                continue;
            }
            float n[3];
            bool fp64;
            if (kPrefix && nprefix && use_cnt <= kSmemHeapMax && kfit <= kSmemHeapMax) {
                // A prefix of at most kSmemHeapMax keys stands for a round the
                // per-lane kernel runs when rounds are not collapsed: it is fitted
                // with that kernel's arithmetic (sums in ascending (d2, index)
                // order), so the normal does not depend on the collapse.
                unsigned long long* sorted = W.keys + (W.cap - kSmemHeapMax);
                wide_sorted_prefix(W, use_cnt, [&](int rank, unsigned long long key) { sorted[rank] = key; });
                __syncwarp();
                float nn[4] = {0.0f, 0.0f, 0.0f, 0.0f};
                if (lane == 0) {
                    const auto point_at = [&](int s) { return neighbour_point(A.T, sorted[s]); };
                    NbrPass P;
                    neighbour_pass<kNem>(point_at, use_cnt, q, P);
                    bool f64 = false;
                    fit_plane<kNem>(A, point_at, use_cnt, q, P, nn, f64);
                    nn[3] = f64 ? 1.0f : 0.0f;
                }
#pragma unroll
                for (int a = 0; a < 3; a++) n[a] = __shfl_sync(kFull, nn[a], 0);
                fp64 = __shfl_sync(kFull, nn[3], 0) != 0.0f;
                __syncwarp();
            } else {
                // Sums in the frame u = (p - q) * 2^-E with |u| < 1 (E from the
                // box), accumulated in 64-bit fixed point: exact and independent
                // of the order in which the search left the neighbours, so every
                // tree layout of the same points gives the same normal.
                const int E = box_exponent(lo, hi, q);
                float mean[3] = {0, 0, 0}, S[6] = {0, 0, 0, 0, 0, 0}, r[6] = {0, 0, 0, 0, 0, 0};
                if (kNem == 2) {
                    long long acc[6] = {0, 0, 0, 0, 0, 0};
                    for (int i = lane; i < cnt; i += 32) {
                        const unsigned long long key = W.keys[i];
                        if (key > use_thr) continue;
                        const float4 p = neighbour_point(A.T, key);
                        const float ux = mul_pow2(__fsub_rn(p.x, q.x), -E), uy = mul_pow2(__fsub_rn(p.y, q.y), -E),
                                    uz = mul_pow2(__fsub_rn(p.z, q.z), -E);
                        acc[0] += to_fixed(__fmul_rn(ux, ux));
                        acc[1] += to_fixed(__fmul_rn(ux, uy));
                        acc[2] += to_fixed(__fmul_rn(ux, uz));
                        acc[3] += to_fixed(__fmul_rn(uy, uy));
                        acc[4] += to_fixed(__fmul_rn(uy, uz));
                        acc[5] += to_fixed(__fmul_rn(uz, uz));
                    }
    #pragma unroll
                    for (int a = 0; a < 6; a++) r[a] = from_fixed(warp_sum_ll(acc[a]));
                } else {
                    long long acc1[3] = {0, 0, 0};
                    for (int i = lane; i < cnt; i += 32) {
                        const unsigned long long key = W.keys[i];
                        if (key > use_thr) continue;
                        const float4 p = neighbour_point(A.T, key);
                        acc1[0] += to_fixed(mul_pow2(__fsub_rn(p.x, q.x), -E));
                        acc1[1] += to_fixed(mul_pow2(__fsub_rn(p.y, q.y), -E));
                        acc1[2] += to_fixed(mul_pow2(__fsub_rn(p.z, q.z), -E));
                    }
                    float su[3], mu[3];
    #pragma unroll
                    for (int a = 0; a < 3; a++) su[a] = from_fixed(warp_sum_ll(acc1[a]));
                    plane_mean<kNem>(su, use_cnt, mu);
                    long long acc[6] = {0, 0, 0, 0, 0, 0};
                    for (int i = lane; i < cnt; i += 32) {
                        const unsigned long long key = W.keys[i];
                        if (key > use_thr) continue;
                        const float4 p = neighbour_point(A.T, key);
                        const float ex = __fsub_rn(mul_pow2(__fsub_rn(p.x, q.x), -E), mu[0]);
                        const float ey = __fsub_rn(mul_pow2(__fsub_rn(p.y, q.y), -E), mu[1]);
                        const float ez = __fsub_rn(mul_pow2(__fsub_rn(p.z, q.z), -E), mu[2]);
                        if (kNem == 3) {
                            acc[0] += to_fixed(__fmul_rn(ex, ex));
                            acc[1] += to_fixed(__fmul_rn(ex, ey));
                            acc[2] += to_fixed(__fmul_rn(ex, ez));
                            acc[3] += to_fixed(__fmul_rn(ey, ey));
                            acc[4] += to_fixed(__fmul_rn(ey, ez));
                            acc[5] += to_fixed(__fmul_rn(ez, ez));
                        } else {
                            acc[0] += to_fixed(__fmul_rn(ex, ex));
                            acc[1] += to_fixed(__fmul_rn(ex, ez));
                            acc[2] += to_fixed(__fmul_rn(ez, ez));
                            acc[3] += to_fixed(__fmul_rn(ex, ey));
                            acc[4] += to_fixed(__fmul_rn(ez, ey));
                        }
                    }
                    // nem 3: the query point's own term (its offset from the mean is -mu)
                    const float own[6] = {__fmul_rn(mu[0], mu[0]), __fmul_rn(mu[0], mu[1]), __fmul_rn(mu[0], mu[2]),
                                          __fmul_rn(mu[1], mu[1]), __fmul_rn(mu[1], mu[2]), __fmul_rn(mu[2], mu[2])};
    #pragma unroll
                    for (int a = 0; a < 6; a++) {
                        const long long own_fx = (kNem == 3) ? to_fixed(own[a]) : 0ll;
                        S[a] = from_fixed(warp_sum_ll(acc[a]) + own_fx);
                    }
                    // the plane offset of nem 0 needs the mean in world units
    #pragma unroll
                    for (int a = 0; a < 3; a++) mean[a] = mul_pow2(mu[a], E);
                }
                solve_plane<kNem>(A.gap_thr, q, mean, S, r, n, fp64);
            }
            // Flip toward the flip point; Normal::operator-() re-normalises.
            const float tx = __fsub_rn(fx, q.x), ty = __fsub_rn(fy, q.y), tz = __fsub_rn(fz, q.z);
            const float dot = __fadd_rn(__fadd_rn(__fmul_rn(n[0], tx), __fmul_rn(n[1], ty)), __fmul_rn(n[2], tz));
            if (dot < 0.0f) {
                n[0] = -n[0]; n[1] = -n[1]; n[2] = -n[2];
                normalize_ieee(n[0], n[1], n[2]);
            }
            if (lane == 0) {
                A.normals[pos] = make_float4(n[0], n[1], n[2], 0.0f);
                if (A.kused) A.kused[pos] = kfit;
                if (fp64) atomicAdd(A.stats + 5, 1u);
                if (nprefix) atomicAdd(A.stats + (fit_round - 1), 1u);
            }
            if (A.nbr) {
                // kNN(ki) of the interpolation = the first ki of this kNN(K >= ki)
                const int m = min(A.ki, use_cnt);
                uint32_t* col = A.nbr + pos;
                const size_t stride = size_t(A.T.n);
                const uint32_t* inv = A.T.inv;
                wide_sorted_prefix(W, m, [&](int rank, unsigned long long key) {
                    col[size_t(rank) * stride] = __ldg(inv + key_idx(key));
                });
                for (int t = m + lane; t < A.ki; t += 32) col[size_t(t) * stride] = 0xffffffffu;
            }
            if (!nprefix) fitted |= 1u << j;
        }
        if (lane == 0 && fitted) atomicAdd(A.stats + (A.round - 1), uint32_t(__popc(fitted)));
        if (lane < nt) A.flags[tile * TQ + lane] = uint8_t((retry >> lane) & 1u);
    }
    if (lane == 0 && st.nodes) {
        atomicAdd(A.stats + 6, st.retries);
        atomicAdd(A.stats + 8, st.buckets);
        atomicAdd(A.stats + 9, st.nodes);
        atomicAdd(A.stats + 13, st.pushes);
        atomicAdd(A.stats + 14, st.chunks);
        atomicAdd(A.stats + 15, st.rounds);
    }
}

// interpolateSurfaceNormals from stored neighbour lists: the same sums as
// interpolate_kernel, in the same order, without a second search.
__global__ void interpolate_lists_kernel(const float4* __restrict__ in, const uint32_t* __restrict__ nbr, int n,
                                         int ki, float4* __restrict__ out, const float4* __restrict__ pad_pts) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= n) return;
    if (pad_pts && __float_as_uint(pad_pts[pos].w) == 0xffffffffu) {
        out[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float4 m = in[pos];
    float x = m.x, y = m.y, z = m.z;
    const int cnt = min(ki, n);
    for (int s = 0; s < cnt; s++) {
        const uint32_t j = __ldg(nbr + size_t(s) * n + pos);
        if (j == 0xffffffffu) break;  // fewer neighbours than ki (a small scan)
        const float4 nj = __ldg(in + j);
        x = __fadd_rn(x, nj.x);
        y = __fadd_rn(y, nj.y);
        z = __fadd_rn(z, nj.z);
    }
    normalize_ieee(x, y, z);
    out[pos] = make_float4(x, y, z, 0.0f);
}

struct InterpArgs {
    Lbvh T;
    int K;
    const float4* in;
    float4* out;
    unsigned long long* gheap;
    int* err;
};

// interpolateSurfaceNormals (AdaptiveKSearchSurface.tcc:293-335)
__global__ void __launch_bounds__(kWarpsPerBlock * 32) interpolate_kernel(InterpArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    for (int tile = blockIdx.x * kWarpsPerBlock + (threadIdx.x >> 5); tile * 32 < A.T.n;
         tile += gridDim.x * kWarpsPerBlock) {
        const int pos = tile * 32 + lane;
        const bool active = pos < A.T.n;
        const float4 q = __ldg(A.T.pts + (active ? pos : 0));
        LaneHeap heap;
        heap.init(ctx.heap, A.K);
        knn_traverse(A.T, q.x, q.y, q.z, active, heap, ctx.stage, A.err, (tile * 32) / A.T.bucket);
        if (active) {
            heap.sort_ascending();
            float4 m = A.in[pos];
            float x = m.x, y = m.y, z = m.z;
            const int cnt = heap.real;
#pragma unroll 4
            for (int s = 0; s < cnt; s++) {
                const unsigned long long key = heap.at(s);
                const float4 nj = __ldg(A.in + __ldg(A.T.inv + key_idx(key)));
                x = __fadd_rn(x, nj.x);
                y = __fadd_rn(y, nj.y);
                z = __fadd_rn(z, nj.z);
            }
            normalize_ieee(x, y, z);
            A.out[pos] = make_float4(x, y, z, 0.0f);
        }
    }
}

struct RowsArgs {
    Lbvh T;
    int K;
    const float4* qs;
    int nq;
    uint32_t* idx;
    float* dist;
    int32_t* count;
    const float4* normals;  // getInterpolatedNormal mode when non-null
    float* nout;
    unsigned long long* gheap;
    int* err;
    float radius2 = INFINITY;  // radius search: only d2 < radius2 (strict)
    int* tiles = nullptr;      // tile counter of a persistent launch
};

template <class Heap>
__device__ __forceinline__ void emit_row(const RowsArgs& A, Heap& heap, float4 q) {
        heap.sort_ascending();
        const size_t row = __float_as_uint(q.w);
        if (A.normals) {
            // PointsetSurface::getInterpolatedNormal: accumulator starts as the
            // default Normal (0, 1, 0); neighbour normals are normalised when
            // read; the sum is divided by ki.  The reference returns
            // Normal<float>(result) with result already a Normal, which is the
            // copy constructor: the mean is not normalised (PointsetSurface.tcc:72-73).
            float x = 0.0f, y = 1.0f, z = 0.0f;
            for (int s = 0; s < A.K; s++) {
                unsigned long long key = heap.at(s);
                if (key == kKeyEmpty) break;
                float4 nj = __ldg(A.normals + __ldg(A.T.inv + key_idx(key)));
                float a = nj.x, b = nj.y, c = nj.z;
                normalize_ieee(a, b, c);
                x = __fadd_rn(x, a);
                y = __fadd_rn(y, b);
                z = __fadd_rn(z, c);
            }
            const float kf = float(A.K);
            x = __fdiv_rn(x, kf);
            y = __fdiv_rn(y, kf);
            z = __fdiv_rn(z, kf);
            A.nout[row * 3 + 0] = x;
            A.nout[row * 3 + 1] = y;
            A.nout[row * 3 + 2] = z;
        } else {
            int c = 0;
            for (int s = 0; s < A.K; s++) {
                unsigned long long key = heap.at(s);
                const bool real = key != kKeyEmpty;
                c += real;
                A.idx[row * A.K + s] = real ? key_idx(key) : 0xffffffffu;
                A.dist[row * A.K + s] = real ? __fsqrt_rn(key_d2(key)) : __int_as_float(0x7f800000);
            }
            if (A.count) A.count[row] = c;
        }
}

template <class Heap>
__global__ void __launch_bounds__(kWarpsPerBlock * 32) rows_kernel(RowsArgs A) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31;
    const WarpCtx ctx = warp_ctx<kWarpsPerBlock>(smem, A.gheap, A.K);
    for (int tile = first_tile<kWarpsPerBlock>(A.tiles); tile * 32 < A.nq;
         tile = next_tile<kWarpsPerBlock>(A.tiles, tile)) {
        const int qi = tile * 32 + lane;
        const bool active = qi < A.nq;
        const float4 q = active ? A.qs[qi] : make_float4(0, 0, 0, 0);
        Heap heap;
        heap.init(ctx.heap, A.K);
        // radius search: keys below (radius2, index 0) are those with d2 < radius2
        if (A.radius2 < FLT_MAX) heap.top = make_key(A.radius2, 0u);
        const float4 q0 = A.qs[tile * 32];
        const int seed = seed_bucket_for(A.T, q0.x, q0.y, q0.z);
        knn_traverse(A.T, q.x, q.y, q.z, active, heap, ctx.stage, A.err, seed);
        if (active) emit_row(A, heap, q);
    }
}

// rows_kernel (index and distance rows) for K > kSmemHeapMax: one warp per
// query (wide.cuh); consecutive Morton-sorted queries of a warp tile chain
// their search bounds as in normals_wide_kernel.
__global__ void __launch_bounds__(kWideWarps * 32, 4) rows_wide_kernel(RowsArgs A, int TQ) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WideState W;
    W.K = A.K;
    W.cap = wide_capacity(A.K);
    W.hist = reinterpret_cast<uint32_t*>(smem) + wib * 256;
    W.keys = A.gheap ? A.gheap + (size_t(blockIdx.x) * kWideWarps + wib) * size_t(W.cap)
                     : reinterpret_cast<unsigned long long*>(smem + kWideWarps * 1024) + size_t(wib) * W.cap;
    const float inf = __int_as_float(0x7f800000);
    // radius search (radius2 > 0): the largest float below radius2, so that
    // d2 <= limit exactly when d2 < radius2
    const float limit = A.radius2 < FLT_MAX ? __int_as_float(__float_as_int(A.radius2) - 1) : inf;
    TravStats st;
    for (int tile = first_tile<kWideWarps>(A.tiles); tile * TQ < A.nq;
         tile = next_tile<kWideWarps>(A.tiles, tile)) {
        const int nt = min(TQ, A.nq - tile * TQ);
        float cx = 0, cy = 0, cz = 0, ctau = inf;
        for (int j = 0; j < nt; j++) {
            const float4 q = A.qs[tile * TQ + j];
            float bound = inf;
            if (ctau < FLT_MAX) {
                const float dx = __fsub_rn(q.x, cx), dy = __fsub_rn(q.y, cy), dz = __fsub_rn(q.z, cz);
                const float delta = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                                         __fmul_rn(dz, dz)));
                const float r = __fmul_rn(__fadd_rn(__fsqrt_rn(ctau), delta), 1.0000038f);
                bound = __fmul_rn(__fmul_rn(r, r), 1.0000038f);
            }
            const int seed = seed_bucket_for(A.T, q.x, q.y, q.z);
            bound = fminf(bound, limit);
            for (int attempt = 0; attempt < 2; attempt++) {
                wide_knn(A.T, q.x, q.y, q.z, W, A.err, st, seed, 0, 0, 0x7fffffff, bound);
                if (W.cnt >= W.K || !(bound < limit)) break;
                bound = limit;
            }
            const int cnt = W.cnt;
            const size_t row = __float_as_uint(q.w);
            uint32_t* ri = A.idx + row * A.K;
            float* rd = A.dist + row * A.K;
            unsigned long long mx = 0;
            for (int i = lane; i < cnt; i += 32) mx = max(mx, W.keys[i]);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(kFull, mx, o));
            wide_sorted_prefix(W, cnt, [&](int r, unsigned long long key) {
                ri[r] = key_idx(key);
                rd[r] = __fsqrt_rn(key_d2(key));
            });
            for (int r = cnt + lane; r < A.K; r += 32) {
                ri[r] = 0xffffffffu;
                rd[r] = inf;
            }
            if (A.count && lane == 0) A.count[row] = cnt;
            ctau = inf;
            if (cnt == W.K) {
                ctau = key_d2(mx);
                cx = q.x; cy = q.y; cz = q.z;
            }
        }
    }
}

__global__ void query_morton_kernel(const float* __restrict__ q, int nq, const float* __restrict__ box,
                                    uint64_t* __restrict__ codes, uint32_t* __restrict__ idx) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const float ext = fmaxf(fmaxf(box[3] - box[0], box[4] - box[1]), box[5] - box[2]);
    codes[i] = morton63(q[3 * size_t(i)], q[3 * size_t(i) + 1], q[3 * size_t(i) + 2], box[0], box[1], box[2],
                        morton_scale(ext));
    idx[i] = uint32_t(i);
}

__global__ void query_gather_kernel(const float* __restrict__ q, const uint32_t* __restrict__ order, int nq,
                                    float4* __restrict__ qs) {
    int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nq) return;
    uint32_t o = order[j];
    qs[j] = make_float4(q[3 * size_t(o)], q[3 * size_t(o) + 1], q[3 * size_t(o) + 2], __uint_as_float(o));
}

// Ordered compaction of a round's retry flags into the next round's query
// list: the list stays in Morton order (consecutive queries of a warp stay
// close in space) and does not depend on the order in which warps finished.
// The query count may live on the device (nq_dev); nq bounds it.
constexpr int kCompactBlock = 1024;

__device__ __forceinline__ int round_count(int nq, const uint32_t* nq_dev) { return nq_dev ? int(*nq_dev) : nq; }

__global__ void __launch_bounds__(kCompactBlock) flag_count_kernel(const uint8_t* __restrict__ flags, int nq,
                                                                   const uint32_t* __restrict__ nq_dev,
                                                                   uint32_t* __restrict__ counts) {
    __shared__ uint32_t part[kCompactBlock / 32];
    const int m = round_count(nq, nq_dev);
    const int i = blockIdx.x * kCompactBlock + threadIdx.x;
    const unsigned b = __ballot_sync(kFull, i < m && flags[i] != 0);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = __popc(b);
    __syncthreads();
    if (threadIdx.x < 32) {
        uint32_t v = part[threadIdx.x];
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(kFull, v, o);
        if (threadIdx.x == 0) counts[blockIdx.x] = v;
    }
}

__global__ void __launch_bounds__(kCompactBlock) flag_scatter_kernel(const uint8_t* __restrict__ flags,
                                                                     const uint32_t* __restrict__ list, int nq,
                                                                     const uint32_t* __restrict__ nq_dev,
                                                                     const uint32_t* __restrict__ offsets,
                                                                     uint32_t* __restrict__ out) {
    __shared__ uint32_t part[kCompactBlock / 32];
    const int m = round_count(nq, nq_dev);
    const int i = blockIdx.x * kCompactBlock + threadIdx.x;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const bool f = i < m && flags[i] != 0;
    const unsigned b = __ballot_sync(kFull, f);
    if (lane == 0) part[w] = __popc(b);
    __syncthreads();
    if (w == 0) {
        const uint32_t v = part[lane];
        uint32_t incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(kFull, incl, o);
            if (lane >= o) incl += t;
        }
        part[lane] = incl - v;
    }
    __syncthreads();
    if (f) out[offsets[blockIdx.x] + part[w] + __popc(b & ((1u << lane) - 1u))] = list ? list[i] : uint32_t(i);
}

int g_num_sms = 0;

template <typename Kernel>
void set_smem(Kernel k, size_t bytes) {
    if (bytes > 48 * 1024) LVRGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(bytes)));
}

// Launches the normals kernel for one search round: per-lane heaps up to
// kSmemHeapMax, one warp per query above.  grid_nq: the number of queries the
// grid is sized for (the round's count, or a cap when the count is on the
// device).
void launch_normals(NormalsArgs& A, int grid_nq, Workspace& ws, cudaStream_t s);

}  // namespace

std::atomic<int> g_round_collapse{1};

int collapse_after_round(int kn, int nem, int adaptive, const uint32_t fitted[5], int64_t n) {
    if (!adaptive || nem == 4 || nem == 1 || !g_round_collapse.load()) return 0;
    if (int64_t(kn) * 32 <= kSmemHeapMax) return 0;  // the last round needs the one-warp-per-query kernel
    int64_t left = n;
    for (int r = 1; r <= 3; r++) {
        const int64_t q = left;  // queries of round r
        left -= int64_t(fitted[r - 1]);
        if (r >= 2 && left > 0 && 10 * int64_t(fitted[r - 1]) < q) return r;
    }
    return 0;
}

HeapPlan plan_heap(int nq, int K, Workspace& ws) {
    if (g_num_sms == 0) {
        int dev = 0;
        LVRGB_CUDA(cudaGetDevice(&dev));
        LVRGB_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    HeapPlan p;
    const int tiles = (nq + 31) / 32;
    const int need_blocks = std::max(1, (tiles + kWarpsPerBlock - 1) / kWarpsPerBlock);
    const size_t stage = size_t(kWarpsPerBlock) * 64 * sizeof(float4);
    if (K <= kSmemHeapMax) {
        p.smem = stage + size_t(kWarpsPerBlock) * K * 32 * sizeof(unsigned long long);
        p.blocks = need_blocks;
        p.gheap = nullptr;
    } else {
        p.smem = stage;
        p.blocks = std::min(need_blocks, g_num_sms * 2);
        p.gheap = ws.get<unsigned long long>("knn.gheap", size_t(p.blocks) * kWarpsPerBlock * K * 32);
    }
    return p;
}

namespace {

// Launch plan of the one-warp-per-query kernels: key buffers in shared
// memory when they fit (200 KB per block), else one global buffer per
// resident warp; long warp tiles carry the chained bound further, shorter
// ones when there are too few queries to give every resident warp work.
struct WidePlan {
    int blocks, tile;
    size_t smem;
    unsigned long long* gbuf;
};
WidePlan plan_wide(int grid_nq, int K, Workspace& ws, int tile_req = 0, int slack = 2) {
    WidePlan P;
    const size_t per_warp = size_t(wide_capacity(K, slack)) * sizeof(unsigned long long);
    P.tile = tile_req > 0 ? std::min(tile_req, kWideTileMax)
                          : std::max(2, std::min(kWideTileMax, grid_nq / (g_num_sms * 128)));
    const int tiles = ceil_div(std::max(grid_nq, 1), P.tile);
    const int need = std::max(1, ceil_div(tiles, kWideWarps));
    P.smem = size_t(kWideWarps) * 1024;
    P.blocks = need;
    P.gbuf = nullptr;
    if (P.smem + kWideWarps * per_warp <= size_t(200) * 1024) {
        P.smem += kWideWarps * per_warp;
    } else {
        const int maxb = int(std::max<size_t>(1, (size_t(1) << 31) / (kWideWarps * per_warp)));
        P.blocks = std::min({need, g_num_sms * 4, maxb});
        P.gbuf = ws.get<unsigned long long>("knn.widebuf", size_t(P.blocks) * kWideWarps * (per_warp / 8));
    }
    return P;
}

// Heap size from which the shared memory limits the per-lane normals kernel
// to five resident blocks (stage + 4 heaps of k keys: 4 KB + 1 KB per key).
constexpr int kFewBlocksK = 36;

template <int kNem>
void launch_normals_nem(NormalsArgs& A, int grid_nq, Workspace& ws, cudaStream_t s) {
    if (A.K <= kSmemHeapMax) {
        HeapPlan P = plan_heap(grid_nq, A.K, ws);
        A.gheap = P.gheap;
        if (A.K == 40) {
            set_smem(normals_kernel<kNem, 5, LaneHeap40>, P.smem);
            A.tiles = persistent_tiles(normals_kernel<kNem, 5, LaneHeap40>, P, ws, s);
            normals_kernel<kNem, 5, LaneHeap40><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
        } else if (A.K >= kFewBlocksK && complete_3ary(A.K)) {
            set_smem(normals_kernel<kNem, 5, LaneHeap3>, P.smem);
            A.tiles = persistent_tiles(normals_kernel<kNem, 5, LaneHeap3>, P, ws, s);
            normals_kernel<kNem, 5, LaneHeap3><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
        } else if (A.K >= kFewBlocksK) {
            set_smem(normals_kernel<kNem, 5>, P.smem);
            A.tiles = persistent_tiles(normals_kernel<kNem, 5>, P, ws, s);
            normals_kernel<kNem, 5><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
        } else {
            // Smaller heaps keep the one-tile-per-warp grid: the persistent
            // form was 2% slower for k = 20 on a 76.5M-point scan project
            // (and faster, 31.8 -> 29.0 ms, for k = 40 on 10M points).
            if (A.K == 20) {
                set_smem(normals_kernel<kNem, 6, LaneHeap20>, P.smem);
                normals_kernel<kNem, 6, LaneHeap20><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
            } else {
                set_smem(normals_kernel<kNem, 6>, P.smem);
                normals_kernel<kNem, 6><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
            }
        }
        A.tiles = nullptr;
        LVRGB_LAUNCH_CHECK();
        return;
    }
    WidePlan P = plan_wide(grid_nq, A.K, ws, A.wide_tile_req, A.wide_slack);
    A.wide_tile = P.tile;
    A.gheap = P.gbuf;
    if (A.nprefix) {
        set_smem(normals_wide_kernel<kNem, true>, P.smem);
        A.tiles = persistent_tiles(normals_wide_kernel<kNem, true>, kWideWarps * 32, P.smem, P.blocks, ws, s);
        normals_wide_kernel<kNem, true><<<P.blocks, kWideWarps * 32, P.smem, s>>>(A);
    } else {
        set_smem(normals_wide_kernel<kNem, false>, P.smem);
        A.tiles = persistent_tiles(normals_wide_kernel<kNem, false>, kWideWarps * 32, P.smem, P.blocks, ws, s);
        normals_wide_kernel<kNem, false><<<P.blocks, kWideWarps * 32, P.smem, s>>>(A);
    }
    A.tiles = nullptr;
    LVRGB_LAUNCH_CHECK();
}

// next[0, *d_count) = the list entries (or, without a list, the indices) of
// [0, count) whose flag is set, in order.  count = *nq_dev when given (then
// nq bounds it), else nq.
void compact_retry(const uint8_t* flags, const uint32_t* list, int nq, const uint32_t* nq_dev, uint32_t* next,
                   uint32_t* d_count, Workspace& ws, cudaStream_t s) {
    const int blocks = std::max(1, ceil_div(nq, kCompactBlock));
    uint32_t* counts = ws.get<uint32_t>("normals.flagcounts", size_t(blocks));
    void* tmp = ws.get<unsigned char>("normals.flagscan", scan_temp_bytes(size_t(blocks)));
    flag_count_kernel<<<blocks, kCompactBlock, 0, s>>>(flags, nq, nq_dev, counts);
    LVRGB_LAUNCH_CHECK();
    exclusive_scan_u32(counts, counts, size_t(blocks), tmp, d_count, s);
    flag_scatter_kernel<<<blocks, kCompactBlock, 0, s>>>(flags, list, nq, nq_dev, counts, next);
    LVRGB_LAUNCH_CHECK();
}

// nem 4 runs with the per-lane heaps only (k <= kSmemHeapMax, checked by the API).
void launch_normals_lbvh(NormalsArgs& A, int grid_nq, Workspace& ws, cudaStream_t s) {
    if (A.K > kSmemHeapMax) throw std::invalid_argument("nem 4 needs k <= 96");
    const HeapPlan P = plan_heap(grid_nq, A.K, ws);
    A.gheap = P.gheap;
    set_smem(normals_kernel<4, 6>, P.smem);
    normals_kernel<4, 6><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    LVRGB_LAUNCH_CHECK();
}

void launch_normals(NormalsArgs& A, int grid_nq, Workspace& ws, cudaStream_t s) {
    if (g_num_sms == 0) {
        int dev = 0;
        LVRGB_CUDA(cudaGetDevice(&dev));
        LVRGB_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    switch (A.nem) {
        case 2: launch_normals_nem<2>(A, grid_nq, ws, s); break;
        case 3: launch_normals_nem<3>(A, grid_nq, ws, s); break;
        case 4: launch_normals_lbvh(A, grid_nq, ws, s); break;
        default: launch_normals_nem<0>(A, grid_nq, ws, s); break;
    }
}

// ---------------------------------------------------------------------------
// nem 1: calcPlaneRANSAC (AdaptiveKSearchSurface.tcc:689-781).
//
// The reference default-constructs its engine on every call and binds copies
// of it and of uniform_int_distribution(0, |id| - 1) (:715-717), so its draws
// depend on the neighbour count m = |id| alone.  Per iteration: draws into an
// unordered_set until it holds three values (at most 21 draws), the set's
// elements in its iteration order, then min(50, m) scoring draws.  The host
// replays them with the same standard-library types (libstdc++, which lvr2
// is built with on Linux) into a schedule; ransac_rows_kernel evaluates the
// iterations per query.  As in the reference, the plane points are
// m_points[r] for the drawn r -- the cloud's points 0..m-1, not the query's
// neighbours (:736-740) -- and the scoring points are the neighbours at the
// drawn ranks (:746-753).  lvr2 reads the `ok` flag without calcPlaneRANSAC
// setting it (:223-231); the RANSAC plane is kept (the other reading of the
// flag is calcPlane, nem 0).
constexpr int kRansacIters = 10;
constexpr int kRansacScore = 50;
constexpr int kRansacStride = 3 + kRansacScore;  // plane draws, then scoring draws

std::vector<uint32_t> ransac_schedule(size_t m) {
    if (m < 3) throw std::invalid_argument("nem 1 needs at least 3 neighbours (kn >= 2 and 3 points)");
    std::vector<uint32_t> out(size_t(kRansacIters) * kRansacStride, 0u);
    std::default_random_engine generator;
    std::uniform_int_distribution<size_t> distribution(0, m - 1);
    auto number = std::bind(distribution, generator);
    std::unordered_set<size_t> ids;
    const int ns = int(std::min<size_t>(kRansacScore, m));
    for (int t = 0; t < kRansacIters; t++) {
        uint32_t* row = out.data() + size_t(t) * kRansacStride;
        ids.clear();
        int c = 0;
        do {
            ids.insert(number());
            c++;
        } while (ids.size() < 3 && c <= 20);
        if (ids.size() < 3)
            throw std::invalid_argument("nem 1: no three distinct plane draws (lvr2 would read past its draw set)");
        auto it = ids.begin();
        for (int j = 0; j < 3; j++, ++it) row[j] = uint32_t(*it);
        for (int j = 0; j < ns; j++) row[3 + j] = uint32_t(number());
    }
    return out;
}

__device__ __forceinline__ float4 point_of(const Lbvh& T, uint32_t orig) { return __ldg(T.pts + __ldg(T.inv + orig)); }

__device__ __forceinline__ float dot_ieee(float ax, float ay, float az, float bx, float by, float bz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(ax, bx), __fmul_rn(ay, by)), __fmul_rn(az, bz));
}

// One thread per query: list[i] = its Morton position, rows + i * K its
// neighbours (original indices, ascending (d2, index)).  Float arithmetic in
// the reference's order: BaseVector cross, Normal normalisation (the null
// vector stays null), dot products left to right.
__global__ void ransac_rows_kernel(Lbvh T, const uint32_t* __restrict__ list, int nq, const uint32_t* __restrict__ rows,
                                   int K, const uint32_t* __restrict__ sched, int ns, float fx, float fy, float fz,
                                   const float4* __restrict__ flip_target, float4* __restrict__ normals,
                                   int* __restrict__ err) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const int pos = int(list[i]);
    const uint32_t* row = rows + size_t(i) * size_t(K);
    float bx = 0.0f, by = 0.0f, bz = 1.0f;  // Normal(0, 0, 1)
    float best = FLT_MAX;
    int nonimproving = 0;
    for (int t = 0; t < kRansacIters && nonimproving < 5; t++) {
        const uint32_t* S = sched + t * kRansacStride;
        const float4 p1 = point_of(T, S[0]), p2 = point_of(T, S[1]), p3 = point_of(T, S[2]);
        const float ux = __fsub_rn(p1.x, p2.x), uy = __fsub_rn(p1.y, p2.y), uz = __fsub_rn(p1.z, p2.z);
        const float vx = __fsub_rn(p1.x, p3.x), vy = __fsub_rn(p1.y, p3.y), vz = __fsub_rn(p1.z, p3.z);
        float nx = __fsub_rn(__fmul_rn(uy, vz), __fmul_rn(uz, vy));
        float ny = __fsub_rn(__fmul_rn(uz, vx), __fmul_rn(ux, vz));
        float nz = __fsub_rn(__fmul_rn(ux, vy), __fmul_rn(uy, vx));
        normalize_ieee(nx, ny, nz);
        const float d1 = dot_ieee(p1.x, p1.y, p1.z, nx, ny, nz);
        float dist = 0.0f;
        for (int j = 0; j < ns; j++) {
            const uint32_t id = row[S[3 + j]];
            if (id >= uint32_t(T.n)) {
                atomicOr(err, kErrRows);
                return;
            }
            const float4 r = point_of(T, id);
            dist = __fadd_rn(dist, fabsf(__fsub_rn(dot_ieee(r.x, r.y, r.z, nx, ny, nz), d1)));
        }
        dist = __fdiv_rn(dist, float(ns));
        if (dist < best) {
            best = dist;
            bx = nx; by = ny; bz = nz;
            nonimproving = 0;
        } else {
            nonimproving++;
        }
    }
    const float4 q = __ldg(T.pts + pos);
    if (flip_target) {
        const float4 t = __ldg(flip_target + pos);
        if (t.w != 0.0f) {
            fx = t.x; fy = t.y; fz = t.z;
        }
    }
    // Flip toward the flip point; Normal::operator-() re-normalises.
    if (dot_ieee(bx, by, bz, __fsub_rn(fx, q.x), __fsub_rn(fy, q.y), __fsub_rn(fz, q.z)) < 0.0f) {
        bx = -bx; by = -by; bz = -bz;
        normalize_ieee(bx, by, bz);
    }
    normals[pos] = make_float4(bx, by, bz, 0.0f);
}

__global__ void kused_flags_kernel(const int32_t* __restrict__ kused, int n, int K, uint8_t* __restrict__ flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) flags[i] = kused[i] == K ? 1 : 0;
}

// Queries at the listed Morton positions, row i tagged in w.
__global__ void list_queries_kernel(const float4* __restrict__ pts, const uint32_t* __restrict__ list, int nq,
                                    float4* __restrict__ qs) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const float4 p = __ldg(pts + list[i]);
    qs[i] = make_float4(p.x, p.y, p.z, __uint_as_float(uint32_t(i)));
}

// Replaces the normals of the points fitted with k = K in the adaptive rounds
// by calcPlaneRANSAC over their sorted K-neighbourhoods.
void ransac_normals(const Lbvh& T, const NormalsConfig& cfg, const int32_t* kused, float4* normals, Workspace& ws,
                    int* d_err, cudaStream_t s) {
    const int n = T.n;
    std::vector<int> ks;
    size_t k = size_t(cfg.kn);
    for (int round = 1; round <= (cfg.adaptive ? 5 : 1); round++) {
        k *= 2;
        ks.push_back(int(std::min<size_t>(k, size_t(1) << 20)));
    }
    const size_t kRowEntries = size_t(1) << 25;  // neighbour entries per chunk (128 MB of indices)
    size_t max_entries = 0;
    for (int K : ks) max_entries = std::max(max_entries, std::min(size_t(n), std::max<size_t>(1, kRowEntries / K)) * K);
    uint8_t* flags = ws.get<uint8_t>("ransac.flags", size_t(n));
    uint32_t* list = ws.get<uint32_t>("ransac.list", size_t(n));
    uint32_t* counter = ws.get<uint32_t>("ransac.count", 1);
    uint32_t* sched = ws.get<uint32_t>("ransac.sched", size_t(kRansacIters) * kRansacStride);
    uint32_t* rows = ws.get<uint32_t>("ransac.rows", max_entries);
    float* dist = ws.get<float>("ransac.dist", max_entries);
    float4* qs = ws.get<float4>("ransac.qs", std::min(size_t(n), max_entries));
    uint64_t* h = ws.pinned();
    for (int K : ks) {
        const size_t m = std::min(size_t(K), size_t(n));
        const std::vector<uint32_t> S = ransac_schedule(m);
        const int ns = int(std::min<size_t>(kRansacScore, m));
        kused_flags_kernel<<<ceil_div(n, 256), 256, 0, s>>>(kused, n, K, flags);
        LVRGB_LAUNCH_CHECK();
        compact_retry(flags, nullptr, n, nullptr, list, counter, ws, s);
        h[0] = 0;
        LVRGB_CUDA(cudaMemcpyAsync(h, counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        LVRGB_CUDA(cudaMemcpyAsync(sched, S.data(), S.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, s));
        LVRGB_CUDA(cudaStreamSynchronize(s));
        const int cnt = int(uint32_t(h[0]));
        const int chunk = int(std::min(size_t(n), std::max<size_t>(1, kRowEntries / K)));
        for (int off = 0; off < cnt; off += chunk) {
            const int c = std::min(chunk, cnt - off);
            list_queries_kernel<<<ceil_div(c, 256), 256, 0, s>>>(T.pts, list + off, c, qs);
            LVRGB_LAUNCH_CHECK();
            knn_rows(T, qs, c, K, rows, dist, nullptr, ws, d_err, s);
            ransac_rows_kernel<<<ceil_div(c, 128), 128, 0, s>>>(T, list + off, c, rows, K, sched, ns, cfg.flip[0],
                                                                cfg.flip[1], cfg.flip[2], cfg.flip_target, normals,
                                                                d_err);
            LVRGB_LAUNCH_CHECK();
        }
    }
}

}  // namespace

void compute_normals(const Lbvh& T, const NormalsConfig& cfg, float4* normals, int32_t* kused, Workspace& ws,
                     int* d_err, uint32_t* d_stats, cudaStream_t s, uint32_t* nbr, int ki) {
    const int n = T.n;
    if (n == 0) return;
    if (cfg.nem == 1 && !kused) kused = ws.get<int32_t>("normals.kused", size_t(n));
    uint32_t* lists[2] = {ws.get<uint32_t>("normals.listA", size_t(n)), ws.get<uint32_t>("normals.listB", size_t(n))};
    uint32_t* counter = ws.get<uint32_t>("normals.counter", 2);
    uint8_t* flags = ws.get<uint8_t>("normals.flags", size_t(n));
    float* kth_d2 = cfg.adaptive ? ws.get<float>("normals.kth", size_t(n)) : nullptr;
    uint64_t* h_count = ws.pinned();
    int nq = n;
    const uint32_t* list = nullptr;
    size_t k = size_t(cfg.kn);
    const bool lbvh = cfg.nem == 4;  // LBVHIndex::knn_normals: one search with k = kn
    bool collapse = false;  // this launch stands in for every remaining round
    for (int round = 1; round <= 5 && nq > 0; round++) {
        if (!lbvh) k *= 2;  // the reference doubles k before every search
        const int round0 = round;
        if (collapse) {
            for (; round < 5; round++) k *= 2;
        }
        const int K = int(std::min<size_t>(k, size_t(1) << 20));
        const int last = (!cfg.adaptive || lbvh || round == 5) ? 1 : 0;
        uint32_t* retry = lists[round & 1];
        NormalsArgs A;
        A.T = T;
        A.K = K;
        A.nem = cfg.nem == 1 ? 0 : cfg.nem;  // nem 1 fits afterwards (ransac_normals)
        A.adaptive = cfg.adaptive;
        A.last_round = last;
        A.round = round;
        A.list = list;
        A.nq = nq;
        A.fx = cfg.flip[0]; A.fy = cfg.flip[1]; A.fz = cfg.flip[2];
        A.gap_thr = cfg.gap_threshold;
        A.normals = normals;
        A.kused = kused;
        A.flags = flags;
        A.kth_d2 = kth_d2;
        A.err = d_err;
        A.stats = d_stats;
        A.nbr = (nbr && ki > 0 && ki <= K) ? nbr : nullptr;
        A.ki = ki;
        A.segs = nullptr;
        A.bucket_scan = nullptr;
        A.nq_dev = nullptr;
        A.flip_target = cfg.flip_target;
        A.wide_tile_req = cfg.wide_tile;
        A.wide_slack = std::max(2, cfg.wide_slack);
        if (collapse) {
            A.nprefix = round - round0;
            A.round_prefix0 = round0;
            for (int p = 0; p < A.nprefix; p++) A.kprefix[p] = int(std::min<size_t>(size_t(cfg.kn) << (round0 + p), size_t(1) << 20));
            A.bound_growth = 1.0f;
            for (int d = round0; d <= round; d++) A.bound_growth *= 2.5f;
        }
        launch_normals(A, nq, ws, s);
        if (last) break;
        compact_retry(flags, list, nq, nullptr, retry, counter, ws, s);
        h_count[0] = 0;
        LVRGB_CUDA(cudaMemcpyAsync(h_count, counter, sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
        LVRGB_CUDA(cudaStreamSynchronize(s));
        const int next = int(uint32_t(h_count[0]));
        // Almost nothing fitted in this round (scans: points on axis-aligned
        // walls and floors fail the box test in every round): search once with
        // the last round's k and test the rounds in between on its prefixes.
        if (cfg.adaptive && !lbvh && cfg.nem != 1 && g_round_collapse.load() && round >= 2 && round <= 3 &&
            next > 0 && 10 * int64_t(nq - next) < int64_t(nq) && int64_t(cfg.kn) * 32 > kSmemHeapMax)
            collapse = true;
        nq = next;
        list = retry;
    }
    // nem 1: the rounds above (run as nem 0) fixed each point's k
    if (cfg.nem == 1) ransac_normals(T, cfg, kused, normals, ws, d_err, s);
}

void compute_normals_segmented(const Lbvh& T, const SegInfo* segs, const uint16_t* bucket_scan,
                               const NormalsConfig& cfg, float4* normals, int32_t* kused, Workspace& ws, int* d_err,
                               uint32_t* d_stats, cudaStream_t s, uint32_t* nbr, int ki, cudaEvent_t* round_ev,
                               int collapse_after) {
    const int n = T.n;
    if (n == 0) return;
    if (g_num_sms == 0) {
        int dev = 0;
        LVRGB_CUDA(cudaGetDevice(&dev));
        LVRGB_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
    }
    uint32_t* lists[2] = {ws.get<uint32_t>("segn.listA", size_t(n)), ws.get<uint32_t>("segn.listB", size_t(n))};
    uint32_t* counters = ws.get<uint32_t>("segn.counters", 8);
    uint8_t* flags = ws.get<uint8_t>("segn.flags", size_t(n));
    float* kth_d2 = cfg.adaptive ? ws.get<float>("segn.kth", size_t(n)) : nullptr;
    LVRGB_CUDA(cudaMemsetAsync(counters, 0, 8 * sizeof(uint32_t), s));
    const bool lbvh = cfg.nem == 4;  // LBVHIndex::knn_normals: one search with k = kn
    const int rounds = (cfg.adaptive && !lbvh) ? 5 : 1;
    if (rounds == 1 || int64_t(cfg.kn) * 32 <= kSmemHeapMax || collapse_after < 2 || collapse_after > 3)
        collapse_after = 0;
    size_t k = size_t(cfg.kn);
    if (round_ev) LVRGB_CUDA(cudaEventRecord(round_ev[0], s));
    for (int round = 1; round <= rounds; round++) {
        if (!lbvh) k *= 2;  // the reference doubles k before every search
        // With collapse_after = r, the launch after round r is the last
        // round's search standing in for rounds r + 1 .. 5.
        const int round0 = round;
        const bool collapse = collapse_after && round == collapse_after + 1;
        if (collapse)
            for (; round < rounds; round++) k *= 2;
        const int K = int(std::min<size_t>(k, size_t(1) << 20));
        NormalsArgs A;
        A.T = T;
        A.K = K;
        A.nem = cfg.nem;
        A.adaptive = cfg.adaptive;
        A.last_round = round == rounds;
        A.round = round;
        A.list = round == 1 ? nullptr : lists[round & 1];
        A.nq = n;
        A.nq_dev = round == 1 ? nullptr : counters + (round - 2);
        A.fx = cfg.flip[0]; A.fy = cfg.flip[1]; A.fz = cfg.flip[2];
        A.gap_thr = cfg.gap_threshold;
        A.normals = normals;
        A.kused = kused;
        A.flags = flags;
        A.kth_d2 = kth_d2;
        A.err = d_err;
        A.stats = d_stats;
        A.nbr = (nbr && ki > 0 && ki <= K) ? nbr : nullptr;
        A.ki = ki;
        A.segs = segs;
        A.bucket_scan = bucket_scan;
        A.flip_target = nullptr;
        A.wide_tile_req = cfg.wide_tile;
        A.wide_slack = std::max(2, cfg.wide_slack);
        if (collapse) {
            // the list and count of the round the collapsed launch starts at
            A.list = lists[round0 & 1];
            A.nq_dev = counters + (round0 - 2);
            A.nprefix = round - round0;
            A.round_prefix0 = round0;
            for (int p = 0; p < A.nprefix; p++) A.kprefix[p] = int(std::min<size_t>(size_t(cfg.kn) << (round0 + p), size_t(1) << 20));
            A.bound_growth = 1.0f;
            for (int d = round0; d <= round; d++) A.bound_growth *= 2.5f;
        }
        // Later rounds read their query count on the device: launch a fixed
        // grid that strides over however many queries the previous round left.
        launch_normals(A, round == 1 ? n : std::min(n, g_num_sms * 8 * kWarpsPerBlock * 32), ws, s);
        if (round < rounds)
            compact_retry(flags, A.list, n, A.nq_dev, lists[(round + 1) & 1], counters + (round - 1), ws, s);
        if (round_ev)
            for (int r = round0; r <= round; r++) LVRGB_CUDA(cudaEventRecord(round_ev[r], s));
    }
    if (round_ev)
        for (int r = rounds + 1; r <= 5; r++) LVRGB_CUDA(cudaEventRecord(round_ev[r], s));
}

void interpolate_normals(const Lbvh& T, int ki, const float4* in, float4* out, Workspace& ws, int* d_err,
                         cudaStream_t s) {
    if (T.n == 0) return;
    if (ki <= 0) {
        LVRGB_CUDA(cudaMemcpyAsync(out, in, sizeof(float4) * size_t(T.n), cudaMemcpyDeviceToDevice, s));
        return;
    }
    InterpArgs A;
    A.T = T;
    A.K = ki;
    A.in = in;
    A.out = out;
    A.err = d_err;
    HeapPlan P = plan_heap(T.n, ki, ws);
    A.gheap = P.gheap;
    set_smem(interpolate_kernel, P.smem);
    interpolate_kernel<<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    LVRGB_LAUNCH_CHECK();
}

void interpolate_from_lists(int n, int ki, const uint32_t* nbr, const float4* in, float4* out, cudaStream_t s,
                            const float4* pad_pts) {
    if (n == 0) return;
    interpolate_lists_kernel<<<ceil_div(n, 256), 256, 0, s>>>(in, nbr, n, ki, out, pad_pts);
    LVRGB_LAUNCH_CHECK();
}

void sort_queries(const float* q, int nq, const float* d_box, float4* qs, Workspace& ws, cudaStream_t s) {
    if (nq == 0) return;
    uint64_t* codes = ws.get<uint64_t>("q.codes", size_t(nq));
    uint64_t* codes2 = ws.get<uint64_t>("q.codes2", size_t(nq));
    uint32_t* idx = ws.get<uint32_t>("q.idx", size_t(nq));
    uint32_t* idx2 = ws.get<uint32_t>("q.idx2", size_t(nq));
    query_morton_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(q, nq, d_box, codes, idx);
    LVRGB_LAUNCH_CHECK();
    void* tmp = ws.get<unsigned char>("q.sorttmp", radix_sort_temp_bytes<uint64_t>(size_t(nq)));
    bool alt = radix_sort_pairs<uint64_t>(codes, idx, codes2, idx2, size_t(nq), 0, 63, tmp, s);
    query_gather_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(q, alt ? idx2 : idx, nq, qs);
    LVRGB_LAUNCH_CHECK();
}

void knn_rows(const Lbvh& T, const float4* qs, int nq, int k, uint32_t* idx, float* dist, int32_t* count,
              Workspace& ws, int* d_err, cudaStream_t s, float radius2) {
    if (nq == 0 || k <= 0) return;
    RowsArgs A;
    A.radius2 = radius2;
    A.T = T;
    A.K = k;
    A.qs = qs;
    A.nq = nq;
    A.idx = idx;
    A.dist = dist;
    A.count = count;
    A.normals = nullptr;
    A.nout = nullptr;
    A.err = d_err;
    if (k > kSmemHeapMax) {
        if (g_num_sms == 0) {
            int dev = 0;
            LVRGB_CUDA(cudaGetDevice(&dev));
            LVRGB_CUDA(cudaDeviceGetAttribute(&g_num_sms, cudaDevAttrMultiProcessorCount, dev));
        }
        WidePlan W = plan_wide(nq, k, ws);
        A.gheap = W.gbuf;
        set_smem(rows_wide_kernel, W.smem);
        A.tiles = persistent_tiles(rows_wide_kernel, kWideWarps * 32, W.smem, W.blocks, ws, s);
        rows_wide_kernel<<<W.blocks, kWideWarps * 32, W.smem, s>>>(A, W.tile);
        LVRGB_LAUNCH_CHECK();
        return;
    }
    HeapPlan P = plan_heap(nq, k, ws);
    A.gheap = P.gheap;
    if (k == 5 && A.radius2 >= FLT_MAX) {
        set_smem(rows_kernel<LaneHeap5>, P.smem);
        A.tiles = persistent_tiles(rows_kernel<LaneHeap5>, P, ws, s);
        rows_kernel<LaneHeap5><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    } else {
        set_smem(rows_kernel<LaneHeap>, P.smem);
        A.tiles = persistent_tiles(rows_kernel<LaneHeap>, P, ws, s);
        rows_kernel<LaneHeap><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    }
    LVRGB_LAUNCH_CHECK();
}

void knn_rows_smem(const Lbvh& T, const float4* qs, int nq, int k, uint32_t* idx, float* dist, int32_t* count,
                   int* d_err, cudaStream_t s) {
    if (nq == 0 || k <= 0) return;
    if (k > kSmemHeapMax) throw std::invalid_argument("k exceeds the shared-memory heap limit");
    RowsArgs A;
    A.T = T;
    A.K = k;
    A.qs = qs;
    A.nq = nq;
    A.idx = idx;
    A.dist = dist;
    A.count = count;
    A.normals = nullptr;
    A.nout = nullptr;
    A.err = d_err;
    A.gheap = nullptr;
    const size_t smem = size_t(kWarpsPerBlock) * 64 * sizeof(float4) +
                        size_t(kWarpsPerBlock) * size_t(k) * 32 * sizeof(unsigned long long);
    const int tiles = (nq + 31) / 32;
    const int blocks = (tiles + kWarpsPerBlock - 1) / kWarpsPerBlock;
    set_smem(rows_kernel<LaneHeap>, smem);
    rows_kernel<LaneHeap><<<blocks, kWarpsPerBlock * 32, smem, s>>>(A);
    LVRGB_LAUNCH_CHECK();
}

void interpolated_normal_rows(const Lbvh& T, const float4* normals, int ki, const float4* qs, int nq, float* out,
                              Workspace& ws, int* d_err, cudaStream_t s) {
    if (nq == 0 || ki <= 0) return;
    RowsArgs A;
    A.T = T;
    A.K = ki;
    A.qs = qs;
    A.nq = nq;
    A.idx = nullptr;
    A.dist = nullptr;
    A.count = nullptr;
    A.normals = normals;
    A.nout = out;
    A.err = d_err;
    HeapPlan P = plan_heap(nq, ki, ws);
    A.gheap = P.gheap;
    set_smem(rows_kernel<LaneHeap>, P.smem);
    rows_kernel<LaneHeap><<<P.blocks, kWarpsPerBlock * 32, P.smem, s>>>(A);
    LVRGB_LAUNCH_CHECK();
}

namespace {
// Largest count and largest used index of neighbour lists (out[0], out[1]).
__global__ void list_extent_kernel(const uint32_t* __restrict__ cnt, const uint32_t* __restrict__ idx, int nq, int k,
                                   uint32_t* __restrict__ out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nq) return;
    const uint32_t c = cnt[i];
    uint32_t m = 0;
    const uint32_t used = c < uint32_t(k) ? c : uint32_t(k);
    for (uint32_t s = 0; s < used; s++) m = max(m, idx[size_t(i) * size_t(k) + s]);
    atomicMax(out, c);
    atomicMax(out + 1, m);
}
}  // namespace

void list_extent(const uint32_t* cnt, const uint32_t* idx, int nq, int k, Workspace& ws, uint32_t out[2],
                 cudaStream_t s) {
    out[0] = out[1] = 0;
    if (nq == 0) return;
    uint32_t* d = ws.get<uint32_t>("lists.extent", 2);
    LVRGB_CUDA(cudaMemsetAsync(d, 0, 2 * sizeof(uint32_t), s));
    list_extent_kernel<<<ceil_div(nq, 256), 256, 0, s>>>(cnt, idx, nq, k, d);
    LVRGB_LAUNCH_CHECK();
    uint64_t* h = ws.pinned();
    LVRGB_CUDA(cudaMemcpyAsync(h, d, 2 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    LVRGB_CUDA(cudaStreamSynchronize(s));
    std::memcpy(out, h, 2 * sizeof(uint32_t));
}

namespace {
// Nearest scan pose of every point (canonical (d2, pose index) order, brute
// force over the poses), and the flip point lvr2 takes from it: the cloud
// point whose input index is the pose's index (m_points[nearestPoseIds[0]],
// AdaptiveKSearchSurface.tcc:255-259).  w = 0 when that index is not a point.
__global__ void pose_target_kernel(Lbvh T, const float* __restrict__ poses, int np, float4* __restrict__ out) {
    const int pos = blockIdx.x * blockDim.x + threadIdx.x;
    if (pos >= T.n) return;
    const float4 q = T.pts[pos];
    unsigned long long best = kKeyEmpty;
    for (int j = 0; j < np; j++) {
        const float d2 = dist2(q.x, q.y, q.z, poses[3 * j], poses[3 * j + 1], poses[3 * j + 2]);
        const unsigned long long key = make_key(d2, uint32_t(j));
        if (key < best) best = key;
    }
    const uint32_t j = key_idx(best);
    if (best == kKeyEmpty || j >= uint32_t(T.n)) {
        out[pos] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    const float4 p = T.pts[T.inv[j]];
    out[pos] = make_float4(p.x, p.y, p.z, 1.0f);
}
}  // namespace

void pose_flip_targets(const Lbvh& T, const float* d_poses, int np, float4* out, cudaStream_t s) {
    if (T.n == 0) return;
    pose_target_kernel<<<ceil_div(T.n, 128), 128, 0, s>>>(T, d_poses, np, out);
    LVRGB_LAUNCH_CHECK();
}

void normals_from_lists(const Lbvh& T, const float* queries, int nq, int k, const uint32_t* cnt, const uint32_t* idx,
                        const float flip[3], float* out, cudaStream_t s) {
    if (nq == 0) return;
    list_normals_kernel<<<ceil_div(nq, 128), 128, 0, s>>>(T, queries, nq, k, cnt, idx, flip[0], flip[1], flip[2], out);
    LVRGB_LAUNCH_CHECK();
}

}  // namespace lvrgb
