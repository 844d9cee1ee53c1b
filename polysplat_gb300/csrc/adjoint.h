// Per-Gaussian forward of the preprocess (raw parameters -> screen centre,
// conic/opacity record, colour) and its adjoint, written once for any
// floating-point type: float in the backward kernel, double in the host-side
// check against finite differences.
//
// The forward follows the same steps as the preprocess kernel:
//   scene transform    opacity = sigmoid(logit), Sigma = R diag(exp(ls))^2 R^T
//                      with R from the normalised w-first quaternion
//                      (csrc/pybind.cpp:22-56)
//   projection         p_hom = proj . [m, 1], xy = ((p_hom.xy / (p_hom.w +
//                      1e-7) + 1) S - 1) / 2 (preprocess.cu:78-81, 360-372)
//   EWA covariance     t = view . [m, 1], tx and ty clamped to 1.3 tan(fov) tz,
//                      J = [[fx/tz, 0, -fx tx/tz^2], [0, fy/tz, -fy ty/tz^2]],
//                      cov2 = J W Sigma W^T J^T + 0.3 I (preprocess.cu:117-157)
//   conic/opacity      (-log2e a/2, -log2e b, -log2e c/2, log2 o) with
//                      (a, b, c) = (cov2.yy, -cov2.xy, cov2.xx) / det
//                      (preprocess.cu:380-395, 624-640)
//   colour             degree-3 SH at dir = (m - campos)/|m - campos|, + 0.5,
//                      clamped at 0 (preprocess.cu:159-255)
// The adjoint differentiates each step exactly (including the clamps: a
// clamped coordinate or colour channel passes no gradient).
#pragma once

#ifdef __CUDACC__
#define GSR_HD __host__ __device__ __forceinline__
#else
#define GSR_HD inline
#include <cmath>
#endif

namespace gsr_adj {

GSR_HD float t_sqrt(float x) { return sqrtf(x); }
GSR_HD double t_sqrt(double x) { return sqrt(x); }
GSR_HD float t_exp(float x) { return expf(x); }
GSR_HD double t_exp(double x) { return exp(x); }
GSR_HD float t_log2(float x) { return log2f(x); }
GSR_HD double t_log2(double x) { return log2(x); }

template <typename T>
struct Cam {
    T view[16];  // column-major world -> view
    T proj[16];  // column-major world -> clip
    T campos[3];
    T fx, fy, tanx, tany;
    int W, H;
};

template <typename T>
struct Fwd {
    T xy[2];
    T con[4];
    T rgb[3];
    T depth;
};

// Basis values B[16] and their gradients dB[16][3] at a unit direction.
template <typename T>
GSR_HD void sh_basis(T x, T y, T z, T B[16], T dB[16][3])
{
    const T C0 = (T)0.28209479177387814, C1 = (T)0.4886025119029199;
    const T c20 = (T)1.0925484305920792, c21 = (T)-1.0925484305920792, c22 = (T)0.31539156525252005,
            c23 = (T)-1.0925484305920792, c24 = (T)0.5462742152960396;
    const T c30 = (T)-0.5900435899266435, c31 = (T)2.890611442640554, c32 = (T)-0.4570457994644658,
            c33 = (T)0.3731763325901154, c34 = (T)-0.4570457994644658, c35 = (T)1.445305721320277,
            c36 = (T)-0.5900435899266435;
    const T xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    B[0] = C0;
    B[1] = -C1 * y;
    B[2] = C1 * z;
    B[3] = -C1 * x;
    B[4] = c20 * xy;
    B[5] = c21 * yz;
    B[6] = c22 * (2 * zz - xx - yy);
    B[7] = c23 * xz;
    B[8] = c24 * (xx - yy);
    B[9] = c30 * y * (3 * xx - yy);
    B[10] = c31 * xy * z;
    B[11] = c32 * y * (4 * zz - xx - yy);
    B[12] = c33 * z * (2 * zz - 3 * xx - 3 * yy);
    B[13] = c34 * x * (4 * zz - xx - yy);
    B[14] = c35 * z * (xx - yy);
    B[15] = c36 * x * (xx - 3 * yy);
    const T d[16][3] = {{0, 0, 0},
                        {0, -C1, 0},
                        {0, 0, C1},
                        {-C1, 0, 0},
                        {c20 * y, c20 * x, 0},
                        {0, c21 * z, c21 * y},
                        {c22 * -2 * x, c22 * -2 * y, c22 * 4 * z},
                        {c23 * z, 0, c23 * x},
                        {c24 * 2 * x, c24 * -2 * y, 0},
                        {c30 * 6 * xy, c30 * (3 * xx - 3 * yy), 0},
                        {c31 * yz, c31 * xz, c31 * xy},
                        {c32 * -2 * xy, c32 * (4 * zz - xx - 3 * yy), c32 * 8 * yz},
                        {c33 * -6 * xz, c33 * -6 * yz, c33 * (6 * zz - 3 * xx - 3 * yy)},
                        {c34 * (4 * zz - 3 * xx - yy), c34 * -2 * xy, c34 * 8 * xz},
                        {c35 * 2 * xz, c35 * -2 * yz, c35 * (xx - yy)},
                        {c36 * (3 * xx - 3 * yy), c36 * -6 * xy, 0}};
    for (int k = 0; k < 16; k++)
        for (int a = 0; a < 3; a++) dB[k][a] = d[k][a];
}

// Rotation matrix (row-major R[i][j]) of a unit w-first quaternion.
template <typename T>
GSR_HD void quat_rot(T r, T x, T y, T z, T R[3][3])
{
    R[0][0] = 1 - 2 * (y * y + z * z);
    R[0][1] = 2 * (x * y - r * z);
    R[0][2] = 2 * (x * z + r * y);
    R[1][0] = 2 * (x * y + r * z);
    R[1][1] = 1 - 2 * (x * x + z * z);
    R[1][2] = 2 * (y * z - r * x);
    R[2][0] = 2 * (x * z - r * y);
    R[2][1] = 2 * (y * z + r * x);
    R[2][2] = 1 - 2 * (x * x + y * y);
}

// Everything the adjoint needs from the forward.
template <typename T>
struct Tape {
    T s[3], qn[4], qlen, R[3][3], Sig[3][3];
    T t[3];
    bool clamp_x, clamp_y;
    T tx, ty;  // the clamped view coordinates
    T J[2][3], A[2][3];
    T a, b, c, det;
    T o;
    T ph[4], w;
    T dir[3], vlen;
    T B[16], dB[16][3];
    bool clamp_rgb[3];
};

template <typename T>
GSR_HD void forward(const T m[3], const T ls[3], const T q[4], T logit, const T* sh, const Cam<T>& cam, Fwd<T>& f,
                    Tape<T>& tp)
{
    // scene transform
    for (int i = 0; i < 3; i++) tp.s[i] = t_exp(ls[i]);
    tp.qlen = t_sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
    for (int i = 0; i < 4; i++) tp.qn[i] = q[i] / tp.qlen;
    quat_rot(tp.qn[0], tp.qn[1], tp.qn[2], tp.qn[3], tp.R);
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            T v = 0;
            for (int k = 0; k < 3; k++) v += tp.R[i][k] * tp.s[k] * tp.s[k] * tp.R[j][k];
            tp.Sig[i][j] = v;
        }
    tp.o = 1 / (1 + t_exp(-logit));
    // view-space position, clamp, Jacobian
    const T* V = cam.view;
    for (int r = 0; r < 3; r++) tp.t[r] = V[r] * m[0] + V[4 + r] * m[1] + V[8 + r] * m[2] + V[12 + r];
    const T limx = (T)1.3 * cam.tanx, limy = (T)1.3 * cam.tany;
    const T tz = tp.t[2];
    const T txtz = tp.t[0] / tz, tytz = tp.t[1] / tz;
    tp.clamp_x = txtz < -limx || txtz > limx;
    tp.clamp_y = tytz < -limy || tytz > limy;
    tp.tx = (tp.clamp_x ? (txtz < 0 ? -limx : limx) : txtz) * tz;
    tp.ty = (tp.clamp_y ? (tytz < 0 ? -limy : limy) : tytz) * tz;
    tp.J[0][0] = cam.fx / tz;
    tp.J[0][1] = 0;
    tp.J[0][2] = -(cam.fx * tp.tx) / (tz * tz);
    tp.J[1][0] = 0;
    tp.J[1][1] = cam.fy / tz;
    tp.J[1][2] = -(cam.fy * tp.ty) / (tz * tz);
    // A = J W, W[r][c] = view rotation (row r) = V[4c + r]
    for (int i = 0; i < 2; i++)
        for (int c = 0; c < 3; c++) tp.A[i][c] = tp.J[i][0] * V[c * 4 + 0] + tp.J[i][1] * V[c * 4 + 1] + tp.J[i][2] * V[c * 4 + 2];
    T C2[2][2];
    for (int i = 0; i < 2; i++)
        for (int j = 0; j < 2; j++) {
            T v = 0;
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) v += tp.A[i][k] * tp.Sig[k][l] * tp.A[j][l];
            C2[i][j] = v;
        }
    const T ca = C2[0][0] + (T)0.3, cb = C2[0][1], cc = C2[1][1] + (T)0.3;
    tp.a = ca;
    tp.b = cb;
    tp.c = cc;
    tp.det = ca * cc - cb * cb;
    const T LOG2E = (T)1.4426950408889634;
    f.con[0] = (T)-0.5 * LOG2E * (cc / tp.det);
    f.con[1] = -LOG2E * (-cb / tp.det);
    f.con[2] = (T)-0.5 * LOG2E * (ca / tp.det);
    f.con[3] = t_log2(tp.o);
    // projection
    const T* P = cam.proj;
    for (int r = 0; r < 4; r++) tp.ph[r] = P[r] * m[0] + P[4 + r] * m[1] + P[8 + r] * m[2] + P[12 + r];
    tp.w = tp.ph[3] + (T)1e-7;
    f.xy[0] = ((tp.ph[0] / tp.w + 1) * cam.W - 1) * (T)0.5;
    f.xy[1] = ((tp.ph[1] / tp.w + 1) * cam.H - 1) * (T)0.5;
    f.depth = tp.t[2];
    // colour
    T v[3] = {m[0] - cam.campos[0], m[1] - cam.campos[1], m[2] - cam.campos[2]};
    tp.vlen = t_sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    for (int i = 0; i < 3; i++) tp.dir[i] = v[i] / tp.vlen;
    sh_basis(tp.dir[0], tp.dir[1], tp.dir[2], tp.B, tp.dB);
    for (int ch = 0; ch < 3; ch++) {
        T r = (T)0.5;
        for (int k = 0; k < 16; k++) r += tp.B[k] * sh[3 * k + ch];
        tp.clamp_rgb[ch] = r < 0;
        f.rgb[ch] = tp.clamp_rgb[ch] ? (T)0 : r;
    }
}

// Gradients of the raw parameters from those of xy, con and rgb.  ADD_SH:
// add the SH gradient to g_sh instead of writing it (a caller summing over
// views needs no second 48-entry array).
template <typename T, bool ADD_SH = false>
GSR_HD void backward(const T m[3], const T* sh, const Cam<T>& cam, const Tape<T>& tp, const T g_xy[2], const T g_con[4],
                     const T g_rgb[3], T g_m[3], T g_ls[3], T g_q[4], T& g_logit, T* g_sh)
{
    const T LOG2E = (T)1.4426950408889634, LN2 = (T)0.6931471805599453;
    for (int i = 0; i < 3; i++) g_m[i] = 0;
    // opacity: con.w = log2(sigmoid(logit))
    g_logit = g_con[3] * (1 - tp.o) / LN2;
    // conic (x, y, z) = (c, -b, a) / det of cov2 (a, b, c)
    const T gx = g_con[0] * (T)-0.5 * LOG2E, gy = g_con[1] * -LOG2E, gz = g_con[2] * (T)-0.5 * LOG2E;
    const T a = tp.a, b = tp.b, c = tp.c, D = tp.det, D2 = D * D;
    const T g_a = (-c * c * gx + b * c * gy - b * b * gz) / D2;
    const T g_b = (2 * b * c * gx + (-D - 2 * b * b) * gy + 2 * a * b * gz) / D2;
    const T g_c = (-b * b * gx + a * b * gy - a * a * gz) / D2;
    // symmetric gradient of cov2 (b counted once over its two entries)
    const T G2[2][2] = {{g_a, g_b / 2}, {g_b / 2, g_c}};
    // dL/dSigma = A^T G2 A
    T GS[3][3];
    for (int k = 0; k < 3; k++)
        for (int l = 0; l < 3; l++) {
            T v = 0;
            for (int i = 0; i < 2; i++)
                for (int j = 0; j < 2; j++) v += tp.A[i][k] * G2[i][j] * tp.A[j][l];
            GS[k][l] = v;
        }
    // dL/dA = 2 G2 A Sigma
    T GA[2][3];
    for (int i = 0; i < 2; i++)
        for (int c2 = 0; c2 < 3; c2++) {
            T v = 0;
            for (int j = 0; j < 2; j++)
                for (int k = 0; k < 3; k++) v += 2 * G2[i][j] * tp.A[j][k] * tp.Sig[k][c2];
            GA[i][c2] = v;
        }
    // A = J W -> dL/dJ = dL/dA W^T, W[r][c] = V[4c + r]
    const T* V = cam.view;
    T GJ[2][3];
    for (int i = 0; i < 2; i++)
        for (int r = 0; r < 3; r++) GJ[i][r] = GA[i][0] * V[0 * 4 + r] + GA[i][1] * V[1 * 4 + r] + GA[i][2] * V[2 * 4 + r];
    // J(t) with the clamps
    const T tz = tp.t[2], tz2 = tz * tz, tz3 = tz2 * tz;
    T g_t[3] = {0, 0, 0};
    g_t[2] += GJ[0][0] * (-cam.fx / tz2) + GJ[1][1] * (-cam.fy / tz2);
    if (tp.clamp_x) {
        g_t[2] += GJ[0][2] * (cam.fx * tp.tx / tz3);  // J02 = -fx lim / tz
    } else {
        g_t[0] += GJ[0][2] * (-cam.fx / tz2);
        g_t[2] += GJ[0][2] * (2 * cam.fx * tp.tx / tz3);
    }
    if (tp.clamp_y) {
        g_t[2] += GJ[1][2] * (cam.fy * tp.ty / tz3);
    } else {
        g_t[1] += GJ[1][2] * (-cam.fy / tz2);
        g_t[2] += GJ[1][2] * (2 * cam.fy * tp.ty / tz3);
    }
    for (int col = 0; col < 3; col++)
        for (int r = 0; r < 3; r++) g_m[col] += V[4 * col + r] * g_t[r];
    // Sigma = R D R^T, D = diag(s^2)
    T RtGR[3];
    for (int k = 0; k < 3; k++) {
        T v = 0;
        for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++) v += tp.R[i][k] * GS[i][j] * tp.R[j][k];
        RtGR[k] = v;
    }
    for (int k = 0; k < 3; k++) g_ls[k] = RtGR[k] * 2 * tp.s[k] * tp.s[k];
    // dL/dR = 2 GS R D
    T GR[3][3];
    for (int i = 0; i < 3; i++)
        for (int k = 0; k < 3; k++) {
            T v = 0;
            for (int j = 0; j < 3; j++) v += GS[i][j] * tp.R[j][k];
            GR[i][k] = 2 * v * tp.s[k] * tp.s[k];
        }
    const T r = tp.qn[0], x = tp.qn[1], y = tp.qn[2], z = tp.qn[3];
    T gqn[4];
    gqn[0] = 2 * (-z * GR[0][1] + y * GR[0][2] + z * GR[1][0] - x * GR[1][2] - y * GR[2][0] + x * GR[2][1]);
    gqn[1] = 2 * (y * GR[0][1] + z * GR[0][2] + y * GR[1][0] - 2 * x * GR[1][1] - r * GR[1][2] + z * GR[2][0] +
                  r * GR[2][1] - 2 * x * GR[2][2]);
    gqn[2] = 2 * (-2 * y * GR[0][0] + x * GR[0][1] + r * GR[0][2] + x * GR[1][0] + z * GR[1][2] - r * GR[2][0] +
                  z * GR[2][1] - 2 * y * GR[2][2]);
    gqn[3] = 2 * (-2 * z * GR[0][0] - r * GR[0][1] + x * GR[0][2] + r * GR[1][0] - 2 * z * GR[1][1] + y * GR[1][2] +
                  x * GR[2][0] + y * GR[2][1]);
    // through the normalisation q / |q|
    const T dq = gqn[0] * tp.qn[0] + gqn[1] * tp.qn[1] + gqn[2] * tp.qn[2] + gqn[3] * tp.qn[3];
    for (int i = 0; i < 4; i++) g_q[i] = (gqn[i] - tp.qn[i] * dq) / tp.qlen;
    // projection
    const T* P = cam.proj;
    T g_ph[4];
    g_ph[0] = g_xy[0] * (T)0.5 * cam.W / tp.w;
    g_ph[1] = g_xy[1] * (T)0.5 * cam.H / tp.w;
    g_ph[2] = 0;
    g_ph[3] = -(g_xy[0] * (T)0.5 * cam.W * tp.ph[0] + g_xy[1] * (T)0.5 * cam.H * tp.ph[1]) / (tp.w * tp.w);
    for (int col = 0; col < 3; col++)
        for (int r4 = 0; r4 < 4; r4++) g_m[col] += P[4 * col + r4] * g_ph[r4];
    // colour
    T g_dir[3] = {0, 0, 0};
    for (int ch = 0; ch < 3; ch++) {
        const T g = tp.clamp_rgb[ch] ? (T)0 : g_rgb[ch];
        for (int k = 0; k < 16; k++) {
            if (ADD_SH) g_sh[3 * k + ch] += tp.B[k] * g;
            else g_sh[3 * k + ch] = tp.B[k] * g;
            for (int d = 0; d < 3; d++) g_dir[d] += tp.dB[k][d] * sh[3 * k + ch] * g;
        }
    }
    const T dd = g_dir[0] * tp.dir[0] + g_dir[1] * tp.dir[1] + g_dir[2] * tp.dir[2];
    for (int i = 0; i < 3; i++) g_m[i] += (g_dir[i] - tp.dir[i] * dd) / tp.vlen;
}

}  // namespace gsr_adj
