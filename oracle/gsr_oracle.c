/*
 * FP64 CPU oracle for the 3DGS forward path -- TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in double precision, the reference rasterizer's
 * algorithm for the hot path (LuoLongZan/PolySplat):
 *
 *   scene transform   csrc/pybind.cpp:22-56, 105-117
 *   view / projection csrc/cuda_rasterizer/preprocess.cu:643-671
 *   preprocess        csrc/cuda_rasterizer/preprocess.cu:78-311, 313-641
 *   tile-key sort     csrc/cuda_rasterizer/sort.cu:14-29, 107-125 (CUB
 *                     DeviceRadixSort::SortPairs semantics: stable,
 *                     ascending, unsigned, over bits [0, end_bit))
 *   tile ranges       csrc/cuda_rasterizer/render.cu:10-35, 3510-3557
 *   feature gather    csrc/cuda_rasterizer/gather.cu:6-22
 *   blend + encode    csrc/cuda_rasterizer/render.cu:228-271, 375-394,
 *                     1783-1858 (whole-tile saturation exit every K)
 *
 * It is only ever called by the test suite, by the smoke check and by the
 * benchmark's CPU-baseline leg; the product path never links it.
 *
 * Parity pinning: the reference ships no golden vectors and no CPU render
 * path.  The oracle is pinned against outputs of the reference's own code
 * run on the same inputs (see tests/golden/), where those exist.
 *
 * Emission order: keys are emitted per Gaussian in index order, tiles in
 * row-major order inside the Gaussian's tile rectangle.  The reference's
 * order is set by atomics and is not deterministic; only sorted outputs
 * are compared, with values compared as multisets inside equal-key runs.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORA_LOG2E 1.4426950216293334961
#define ORA_LN2 0.69314718055

/* SH basis constants, preprocess.cu:25-38 */
static const double C0 = 0.28209479177387814;
static const double C1 = 0.4886025119029199;
static const double C2[5] = {1.0925484305920792, -1.0925484305920792, 0.31539156525252005,
                             -1.0925484305920792, 0.5462742152960396};
static const double C3[7] = {-0.5900435899266435, 2.890611442640554, -0.4570457994644658,
                             0.3731763325901154, -0.4570457994644658, 1.445305721320277,
                             -0.5900435899266435};

/* ------------------------------------------------------------------------- */
/* Scene transform: pybind.cpp:105-117 (sigmoid, exp, normalise) and
 * computeCov3D pybind.cpp:22-56 (Sigma = R S^2 R^T, upper triangle). */
void ora_scene_transform(int P, const float* log_scales, const float* quats,
                         const float* logits, float* opacity, float* cov3d)
{
    for (int i = 0; i < P; i++) {
        opacity[i] = (float)(1.0 / (1.0 + exp(-(double)logits[i])));
        double s[3];
        for (int k = 0; k < 3; k++) s[k] = exp((double)log_scales[3 * i + k]);
        double q[4];
        double n = 0.0;
        for (int k = 0; k < 4; k++) { q[k] = quats[4 * i + k]; n += q[k] * q[k]; }
        n = sqrt(n);
        for (int k = 0; k < 4; k++) q[k] /= n;
        double r = q[0], x = q[1], y = q[2], z = q[3];
        /* standard rotation matrix of the w-first quaternion (row major) */
        double R[3][3] = {
            {1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)},
            {2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)},
            {2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)}};
        double S[3][3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0.0;
                for (int k = 0; k < 3; k++) acc += R[a][k] * s[k] * s[k] * R[b][k];
                S[a][b] = acc;
            }
        float* c = cov3d + 6 * i;
        c[0] = (float)S[0][0]; c[1] = (float)S[0][1]; c[2] = (float)S[0][2];
        c[3] = (float)S[1][1]; c[4] = (float)S[1][2]; c[5] = (float)S[2][2];
    }
}

/* ------------------------------------------------------------------------- */
/* Camera: getViewMatrix / getProjectionMatrix, preprocess.cu:643-671.
 * rot is the row-major 3x3 tensor handed to the op; its rows become the
 * columns of the glm matrix (pybind.cpp:141-143), so world->view is rot^T. */
typedef struct {
    double view[3][4];  /* rows: x, y, z of view space */
    double proj[4][4];  /* full projection (row major) */
    double campos[3];
} ora_cam;

static void make_cam(ora_cam* c, int W, int H, const float* pos, const float* rot,
                     double fx, double fy, double zfar, double znear)
{
    /* M[r][k] = rot[k][r] */
    double M[3][3];
    for (int r = 0; r < 3; r++)
        for (int k = 0; k < 3; k++) M[r][k] = rot[3 * k + r];
    for (int r = 0; r < 3; r++) {
        double t = 0.0;
        for (int k = 0; k < 3; k++) { c->view[r][k] = M[r][k]; t -= M[r][k] * pos[k]; }
        c->view[r][3] = t;
        c->campos[r] = pos[r];
    }
    double top = H / (2.0 * fy) * znear, bottom = -top;
    double right = W / (2.0 * fx) * znear, left = -right;
    double Pm[4][4];
    memset(Pm, 0, sizeof Pm);
    /* glm P[col][row]; after transpose(P) the math matrix has these rows */
    Pm[0][0] = 2.0 * znear / (right - left);
    Pm[1][1] = 2.0 * znear / (top - bottom);
    Pm[0][2] = (right + left) / (right - left);
    Pm[1][2] = (top + bottom) / (top - bottom);
    Pm[3][2] = 1.0;
    Pm[2][2] = zfar / (zfar - znear);
    Pm[2][3] = -(zfar * znear) / (zfar - znear);
    double V4[4][4] = {{0}};
    for (int r = 0; r < 3; r++)
        for (int k = 0; k < 4; k++) V4[r][k] = c->view[r][k];
    V4[3][3] = 1.0;
    for (int r = 0; r < 4; r++)
        for (int k = 0; k < 4; k++) {
            double acc = 0.0;
            for (int j = 0; j < 4; j++) acc += Pm[r][j] * V4[j][k];
            c->proj[r][k] = acc;
        }
}

/* ------------------------------------------------------------------------- */
/* Tile tests, preprocess.cu:257-311 */
static int seg_intersect(double a, double b, double c, double d, double l, double r)
{
    double delta = b * b - 4.0 * a * c;
    double t1 = (l - d) * (2.0 * a) + b;
    double t2 = (r - d) * (2.0 * a) + b;
    return delta >= 0.0 && (t1 <= 0.0 || t1 * t1 <= delta) && (t2 >= 0.0 || t2 * t2 <= delta);
}

static int block_intersect(int pminx, int pminy, int pmaxx, int pmaxy, double cx, double cy,
                           const double con[3], double power)
{
    double w = 2.0 * power, dx, dy;
    dx = (cx * 2.0 < pminx + pmaxx) ? cx - pminx : cx - pmaxx;
    if (seg_intersect(con[2], -2.0 * con[1] * dx, con[0] * dx * dx - w, cy, pminy, pmaxy)) return 1;
    dy = (cy * 2.0 < pminy + pmaxy) ? cy - pminy : cy - pmaxy;
    if (seg_intersect(con[0], -2.0 * con[1] * dy, con[2] * dy * dy - w, cx, pminx, pmaxx)) return 1;
    return 0;
}

static int block_contains(int pminx, int pminy, int pmaxx, int pmaxy, double cx, double cy)
{
    return cx >= pminx && cx <= pmaxx && cy >= pminy && cy <= pmaxy;
}

static int imin(int a, int b) { return a < b ? a : b; }
static int imax(int a, int b) { return a > b ? a : b; }

/* Per-Gaussian geometry shared by the emission and feature passes. */
typedef struct {
    int valid;
    int rminx, rminy, rmaxx, rmaxy;
    double px, py, depth, power, log2o;
    double con[3];
} ora_geom;

static void gauss_geom(const ora_cam* c, int W, int H, int bx, int by, int gx, int gy,
                       double tanx, double tany, double fx, double fy,
                       const float* p3, float o, const float* cv, ora_geom* g)
{
    memset(g, 0, sizeof *g);
    double p[3] = {p3[0], p3[1], p3[2]};
    double t[3];
    for (int r = 0; r < 3; r++)
        t[r] = c->view[r][0] * p[0] + c->view[r][1] * p[1] + c->view[r][2] * p[2] + c->view[r][3];
    if (t[2] <= 0.2) return;                                     /* :363 */
    double hom[4];
    for (int r = 0; r < 4; r++)
        hom[r] = c->proj[r][0] * p[0] + c->proj[r][1] * p[1] + c->proj[r][2] * p[2] + c->proj[r][3];
    double pw = 1.0 / (hom[3] + 0.0000001);                      /* :375 */
    double ndx = hom[0] * pw, ndy = hom[1] * pw;
    /* computeCov2D, preprocess.cu:117-157 */
    double limx = 1.3 * tanx, limy = 1.3 * tany;
    double txtz = t[0] / t[2], tytz = t[1] / t[2];
    double tx = fmin(limx, fmax(-limx, txtz)) * t[2];
    double ty = fmin(limy, fmax(-limy, tytz)) * t[2];
    double tz = t[2];
    double J[2][3] = {{fx / tz, 0.0, -(fx * tx) / (tz * tz)}, {0.0, fy / tz, -(fy * ty) / (tz * tz)}};
    /* T = J * Wv  (Wv = upper 3x3 of view), cov = T Sigma T^T */
    double Tm[2][3];
    for (int a = 0; a < 2; a++)
        for (int k = 0; k < 3; k++)
            Tm[a][k] = J[a][0] * c->view[0][k] + J[a][1] * c->view[1][k] + J[a][2] * c->view[2][k];
    double Sg[3][3] = {{cv[0], cv[1], cv[2]}, {cv[1], cv[3], cv[4]}, {cv[2], cv[4], cv[5]}};
    double cov[2][2];
    for (int a = 0; a < 2; a++)
        for (int b = 0; b < 2; b++) {
            double acc = 0.0;
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) acc += Tm[a][k] * Sg[k][l] * Tm[b][l];
            cov[a][b] = acc;
        }
    double cxx = cov[0][0] + 0.3, cxy = cov[0][1], cyy = cov[1][1] + 0.3;
    double det = cxx * cyy - cxy * cxy;
    double di = 1.0 / det;
    g->con[0] = cyy * di; g->con[1] = -cxy * di; g->con[2] = cxx * di;
    g->log2o = log2((double)o);
    g->power = ORA_LN2 * 8.0 + ORA_LN2 * g->log2o;               /* :391-392 */
    double trace = cxx + cyy;
    if (2.0 * det * g->power < 0.09 * trace && o < 0.5) return;  /* :396-398 */
    int w = (int)(1.414214 * sqrt(cxx * g->power) + 1.0);          /* :401-402 */
    int h = (int)(1.414214 * sqrt(cyy * g->power) + 1.0);
    g->px = ((ndx + 1.0) * W - 1.0) * 0.5;                        /* ndc2Pix :78-81 */
    g->py = ((ndy + 1.0) * H - 1.0) * 0.5;
    /* getRect, preprocess.cu:104-114 (the reference truncates in float) */
    double fpx = (float)g->px, fpy = (float)g->py;
    g->rminx = imin(gx, imax(0, (int)((fpx - w) / bx)));
    g->rminy = imin(gy, imax(0, (int)((fpy - h) / by)));
    g->rmaxx = imin(gx, imax(0, (int)((fpx + w) / bx) + 1));
    g->rmaxy = imin(gy, imax(0, (int)((fpy + h) / by) + 1));
    g->depth = t[2];
    g->valid = (g->rmaxx - g->rminx) * (g->rmaxy - g->rminy) > 0;
}

static int tile_hit(const ora_geom* g, int x, int y, int bx, int by)
{
    int pminx = x * bx, pminy = y * by;
    int pmaxx = pminx + bx - 1, pmaxy = pminy + by - 1;
    double cx = (float)g->px, cy = (float)g->py;
    return block_contains(pminx, pminy, pmaxx, pmaxy, cx, cy) ||
           (g->power > 0.0 && block_intersect(pminx, pminy, pmaxx, pmaxy, cx, cy, g->con, g->power));
}

static void sh_color(const double dir_in[3], const float* sh, double rgb[3])
{
    double l = sqrt(dir_in[0] * dir_in[0] + dir_in[1] * dir_in[1] + dir_in[2] * dir_in[2]);
    double x = dir_in[0] / l, y = dir_in[1] / l, z = dir_in[2] / l;
    double xx = x * x, yy = y * y, zz = z * z, xy = x * y, yz = y * z, xz = x * z;
    double basis[16] = {
        C0, -C1 * y, C1 * z, -C1 * x,
        C2[0] * xy, C2[1] * yz, C2[2] * (2.0 * zz - xx - yy), C2[3] * xz, C2[4] * (xx - yy),
        C3[0] * y * (3.0 * xx - yy), C3[1] * xy * z, C3[2] * y * (4.0 * zz - xx - yy),
        C3[3] * z * (2.0 * zz - 3.0 * xx - 3.0 * yy), C3[4] * x * (4.0 * zz - xx - yy),
        C3[5] * z * (xx - yy), C3[6] * x * (xx - 3.0 * yy)};
    for (int ch = 0; ch < 3; ch++) {
        double acc = 0.0;
        for (int k = 0; k < 16; k++) acc += basis[k] * sh[3 * k + ch];
        acc += 0.5;                                  /* :170 */
        rgb[ch] = acc > 0.0 ? acc : 0.0;             /* :195-197, no upper clamp */
    }
}

/* preprocess.cu:313-641.  Writes features for every Gaussian that emitted
 * at least one key (emitted[i] = 1) and the (key, value) list.  Returns the
 * true number of keys (may exceed capacity; writes are clamped).  The work
 * is split into contiguous Gaussian chunks, one per thread: a counting pass,
 * a prefix sum, then an emission pass, so the key order is the same for any
 * thread count. */
typedef struct {
    const ora_cam* c;
    int P0, P1, W, H, bx, by, gx, gy;
    double tanx, tany, fx, fy;
    const float *pos, *shs, *opacity, *cov3d;
    float *points_xy, *rgb_depth, *conic_opacity;
    uint8_t* emitted;
    uint64_t* keys;
    uint32_t* vals;
    int64_t capacity, base, count;
    int emit;
} ora_pre_job;

static void* pre_worker(void* arg)
{
    ora_pre_job* j = (ora_pre_job*)arg;
    int64_t m = j->base;
    for (int i = j->P0; i < j->P1; i++) {
        ora_geom g;
        gauss_geom(j->c, j->W, j->H, j->bx, j->by, j->gx, j->gy, j->tanx, j->tany, j->fx, j->fy,
                   j->pos + 3 * (size_t)i, j->opacity[i], j->cov3d + 6 * (size_t)i, &g);
        if (j->emit) j->emitted[i] = 0;
        if (!g.valid) continue;
        float fd = (float)g.depth;
        uint32_t dbits;
        memcpy(&dbits, &fd, 4);
        int hit_any = 0;
        for (int y = g.rminy; y < g.rmaxy; y++)
            for (int x = g.rminx; x < g.rmaxx; x++) {
                if (!tile_hit(&g, x, y, j->bx, j->by)) continue;
                if (j->emit && m < j->capacity) {
                    j->keys[m] = ((uint64_t)(uint32_t)(y * j->gx + x) << 32) | dbits;
                    j->vals[m] = (uint32_t)i;
                }
                m++;
                hit_any = 1;
            }
        if (j->emit && hit_any) {
            const ora_cam* c = j->c;
            const float* p = j->pos + 3 * (size_t)i;
            double dir[3] = {p[0] - c->campos[0], p[1] - c->campos[1], p[2] - c->campos[2]};
            double rgb[3];
            sh_color(dir, j->shs + 48 * (size_t)i, rgb);
            j->emitted[i] = 1;
            j->points_xy[2 * (size_t)i] = (float)g.px;
            j->points_xy[2 * (size_t)i + 1] = (float)g.py;
            float* rd = j->rgb_depth + 4 * (size_t)i;
            rd[0] = (float)rgb[0]; rd[1] = (float)rgb[1]; rd[2] = (float)rgb[2]; rd[3] = fd;
            float* co = j->conic_opacity + 4 * (size_t)i;
            co[0] = (float)(-0.5 * ORA_LOG2E * g.con[0]);   /* :627 */
            co[1] = (float)(-ORA_LOG2E * g.con[1]);
            co[2] = (float)(-0.5 * ORA_LOG2E * g.con[2]);
            co[3] = (float)g.log2o;
        }
    }
    j->count = m - j->base;
    return NULL;
}

int64_t ora_preprocess(int P, const float* pos, const float* shs, const float* opacity,
                       const float* cov3d, int W, int H, int bx, int by,
                       const float* cam_pos, const float* cam_rot, float fx, float fy,
                       float zfar, float znear,
                       float* points_xy, float* rgb_depth, float* conic_opacity, uint8_t* emitted,
                       uint64_t* keys, uint32_t* vals, int64_t capacity, int nthreads)
{
    ora_cam c;
    make_cam(&c, W, H, cam_pos, cam_rot, fx, fy, zfar, znear);
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    ora_pre_job jobs[256];
    int chunk = (P + nthreads - 1) / nthreads;
    for (int t = 0; t < nthreads; t++) {
        ora_pre_job* j = &jobs[t];
        j->c = &c;
        j->P0 = imin(P, t * chunk); j->P1 = imin(P, (t + 1) * chunk);
        j->W = W; j->H = H; j->bx = bx; j->by = by;
        j->gx = (W + bx - 1) / bx; j->gy = (H + by - 1) / by;
        j->tanx = W / (2.0 * fx); j->tany = H / (2.0 * fy); j->fx = fx; j->fy = fy;
        j->pos = pos; j->shs = shs; j->opacity = opacity; j->cov3d = cov3d;
        j->points_xy = points_xy; j->rgb_depth = rgb_depth; j->conic_opacity = conic_opacity;
        j->emitted = emitted; j->keys = keys; j->vals = vals; j->capacity = capacity;
        j->base = 0; j->emit = 0;
    }
    for (int pass = 0; pass < 2; pass++) {
        for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, pre_worker, &jobs[t]);
        pre_worker(&jobs[0]);
        for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);
        if (pass == 0) {
            int64_t acc = 0;
            for (int t = 0; t < nthreads; t++) { jobs[t].base = acc; acc += jobs[t].count; jobs[t].emit = 1; }
        }
    }
    int64_t total = 0;
    for (int t = 0; t < nthreads; t++) total += jobs[t].count;
    return total;
}

/* ------------------------------------------------------------------------- */
/* sort.cu:14-29: number of bits needed for n (binary search formulation). */
uint32_t ora_higher_msb(uint32_t n)
{
    uint32_t msb = sizeof(n) * 4;
    uint32_t step = msb;
    while (step > 1) {
        step /= 2;
        if (n >> msb) msb += step; else msb -= step;
    }
    if (n >> msb) msb++;
    return msb;
}

/* Stable ascending LSD radix sort over bits [0, end_bit) of u64 keys with u32
 * payloads: the contract of cub::DeviceRadixSort::SortPairs (sort.cu:116-120).
 * Bits at or above end_bit are carried but ignored for ordering. */
void ora_sort_pairs(int64_t n, const uint64_t* kin, const uint32_t* vin, uint64_t* kout,
                    uint32_t* vout, int end_bit)
{
    size_t cap = (size_t)(n ? n : 1);
    uint64_t* ka = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    uint32_t* va = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    uint64_t* kb = (uint64_t*)malloc(sizeof(uint64_t) * cap);
    uint32_t* vb = (uint32_t*)malloc(sizeof(uint32_t) * cap);
    memcpy(ka, kin, sizeof(uint64_t) * n);
    memcpy(va, vin, sizeof(uint32_t) * n);
    int passes = (end_bit + 7) / 8;
    for (int p = 0; p < passes; p++) {
        int shift = 8 * p;
        int bits = end_bit - shift < 8 ? end_bit - shift : 8;
        uint64_t mask = ((uint64_t)1 << bits) - 1;
        int64_t cnt[257];
        memset(cnt, 0, sizeof cnt);
        for (int64_t i = 0; i < n; i++) cnt[((ka[i] >> shift) & mask) + 1]++;
        for (int d = 0; d < 256; d++) cnt[d + 1] += cnt[d];
        for (int64_t i = 0; i < n; i++) {
            uint64_t d = (ka[i] >> shift) & mask;
            int64_t o = cnt[d]++;
            kb[o] = ka[i];
            vb[o] = va[i];
        }
        uint64_t* tk = ka; ka = kb; kb = tk;
        uint32_t* tv = va; va = vb; vb = tv;
    }
    memcpy(kout, ka, sizeof(uint64_t) * n);
    memcpy(vout, va, sizeof(uint32_t) * n);
    free(ka); free(va); free(kb); free(vb);
}

/* ------------------------------------------------------------------------- */
/* render.cu:10-35 + 3510-3521: [lower_bound, upper_bound) per tile. */
void ora_tile_ranges_bsearch(int64_t n, const uint64_t* keys, int tiles, int32_t* ranges)
{
    for (int t = 0; t < tiles; t++) {
        int64_t lo = 0, hi = n;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((keys[mid] >> 32) < (uint64_t)t) lo = mid + 1; else hi = mid;
        }
        int64_t start = lo;
        hi = n;
        while (lo < hi) {
            int64_t mid = (lo + hi) >> 1;
            if ((keys[mid] >> 32) <= (uint64_t)t) lo = mid + 1; else hi = mid;
        }
        ranges[2 * t] = (int32_t)start;
        ranges[2 * t + 1] = (int32_t)lo;
    }
}

/* render.cu:3526-3557 (after the zero fill of render.cu:6838). */
void ora_tile_ranges_scan(int64_t n, const uint64_t* keys, int tiles, int32_t* ranges)
{
    memset(ranges, 0, sizeof(int32_t) * 2 * (size_t)tiles);
    for (int64_t i = 0; i < n; i++) {
        uint32_t cur = (uint32_t)(keys[i] >> 32);
        if (i == 0) ranges[2 * cur] = 0;
        else {
            uint32_t prev = (uint32_t)(keys[i - 1] >> 32);
            if (cur != prev) { ranges[2 * prev + 1] = (int32_t)i; ranges[2 * cur] = (int32_t)i; }
        }
        if (i == n - 1) ranges[2 * cur + 1] = (int32_t)n;
    }
}

/* gather.cu:6-22 */
void ora_gather(int64_t n, const uint32_t* vals, const float* xy, const float* rgbd, const float* con,
                float* dxy, float* drgbd, float* dcon)
{
    for (int64_t i = 0; i < n; i++) {
        uint32_t g = vals[i];
        memcpy(dxy + 2 * i, xy + 2 * (size_t)g, 8);
        memcpy(drgbd + 4 * i, rgbd + 4 * (size_t)g, 16);
        memcpy(dcon + 4 * i, con + 4 * (size_t)g, 16);
    }
}

/* ------------------------------------------------------------------------- */
/* Blend, render.cu:228-271 (pixel_shader_axis_shared_16x16), 375-394
 * (encode/write_color), 1783-1858 (whole-tile saturation exit).  `cadence`
 * is the exit-check period: after the j-th Gaussian of a tile (1-based),
 * when j % cadence == 0 and every pixel of the tile (including those outside
 * the image) has T < 1e-4, the tile stops.  dt != 0 reproduces the
 * "_dt" variant that skips contributions with power < log2(1/255). */
typedef struct {
    int64_t n;
    const uint32_t* vals;
    const int32_t* ranges;
    const float* xy;
    const float* rgbd;
    const float* con;
    int W, H, bx, by, gx, tiles, cadence, dt;
    double bg[3];
    uint8_t* out;
    int64_t* contrib;   /* optional per-tile count of Gaussians processed */
    int nthreads, tid;
} ora_render_job;

static uint8_t encode(double x)
{
    double v = x * 255.0;
    if (v < 0.0) v = 0.0;
    if (v > 255.0) v = 255.0;
    return (uint8_t)v;
}

static void* render_worker(void* arg)
{
    ora_render_job* j = (ora_render_job*)arg;
    int npx = j->bx * j->by;
    double* T = (double*)malloc(sizeof(double) * npx);
    double* C = (double*)malloc(sizeof(double) * npx * 3);
    for (int t = j->tid; t < j->tiles; t += j->nthreads) {
        int ox = (t % j->gx) * j->bx, oy = (t / j->gx) * j->by;
        int32_t s = j->ranges[2 * t], e = j->ranges[2 * t + 1];
        for (int p = 0; p < npx; p++) { T[p] = 1.0; C[3 * p] = C[3 * p + 1] = C[3 * p + 2] = 0.0; }
        int64_t processed = 0;
        for (int32_t k = s; k < e; k++) {
            uint32_t g = j->vals[k];
            const float* xy = j->xy + 2 * (size_t)g;
            const float* cr = j->rgbd + 4 * (size_t)g;
            const float* co = j->con + 4 * (size_t)g;
            for (int p = 0; p < npx; p++) {
                double dx = xy[0] - (double)(ox + p % j->bx);
                double dy = xy[1] - (double)(oy + p / j->bx);
                double power = co[3] + co[0] * dx * dx + co[2] * dy * dy + co[1] * dx * dy;
                if (j->dt && power < -7.994353375) continue;
                double a = exp2(power);
                double w = a * T[p];
                C[3 * p] += cr[0] * w;
                C[3 * p + 1] += cr[1] * w;
                C[3 * p + 2] += cr[2] * w;
                T[p] -= w;
            }
            processed++;
            if (processed % j->cadence == 0) {
                int sat = 1;
                for (int p = 0; p < npx && sat; p++) sat = T[p] < 0.0001;
                if (sat) break;
            }
        }
        if (j->contrib) j->contrib[t] = processed;
        for (int p = 0; p < npx; p++) {
            int px = ox + p % j->bx, py = oy + p / j->bx;
            if (px >= j->W || py >= j->H) continue;
            uint8_t* o = j->out + 3 * ((size_t)py * j->W + px);
            if (e - s <= 0) {
                for (int ch = 0; ch < 3; ch++) o[ch] = encode(j->bg[ch]);
            } else {
                double tt = T[p] < 0.0001 ? 0.0 : T[p];
                for (int ch = 0; ch < 3; ch++) o[ch] = encode(C[3 * p + ch] + tt * j->bg[ch]);
            }
        }
    }
    free(T);
    free(C);
    return NULL;
}

void ora_render(int64_t n, const uint32_t* vals, const int32_t* ranges, const float* xy,
                const float* rgbd, const float* con, int W, int H, int bx, int by, int cadence,
                int dt, const float* bg, uint8_t* out, int64_t* contrib, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    ora_render_job jobs[256];
    int gx = (W + bx - 1) / bx, gy = (H + by - 1) / by;
    for (int i = 0; i < nthreads; i++) {
        ora_render_job* j = &jobs[i];
        j->n = n; j->vals = vals; j->ranges = ranges; j->xy = xy; j->rgbd = rgbd; j->con = con;
        j->W = W; j->H = H; j->bx = bx; j->by = by; j->gx = gx; j->tiles = gx * gy;
        j->cadence = cadence > 0 ? cadence : 1; j->dt = dt;
        for (int ch = 0; ch < 3; ch++) j->bg[ch] = bg[ch];
        j->out = out; j->contrib = contrib; j->nthreads = nthreads; j->tid = i;
    }
    for (int i = 1; i < nthreads; i++) pthread_create(&th[i], NULL, render_worker, &jobs[i]);
    render_worker(&jobs[0]);
    for (int i = 1; i < nthreads; i++) pthread_join(th[i], NULL);
}

/* ------------------------------------------------------------------------- */
/* Differentiable-render reference (test infrastructure): the float image of
 * one camera computed in double end to end from the raw parameters (means,
 * log-scales, w-first quaternions, opacity logits, SH), with the tile
 * emission, (tile, depth) order and whole-tile saturation exit of the
 * forward (the same rules as ora_preprocess / ora_render, every continuous
 * quantity in double).  The L2 loss against `target` is returned, so central
 * differences of it check the gradients of the CUDA backward.  Tiles are
 * rendered by nthreads threads; the result does not depend on the count. */
typedef struct {
    double px, py, depth, con[3], log2o, rgb[3], power;
    int x0, y0, x1, y1;  /* tile rectangle */
    int ok;
} ora_dg;

typedef struct {
    uint32_t tile;
    double depth;
    uint32_t gid;
} ora_pair;

static int pair_cmp(const void* a, const void* b)
{
    const ora_pair* x = (const ora_pair*)a;
    const ora_pair* y = (const ora_pair*)b;
    if (x->tile != y->tile) return x->tile < y->tile ? -1 : 1;
    if (x->depth != y->depth) return x->depth < y->depth ? -1 : 1;
    return x->gid < y->gid ? -1 : (x->gid > y->gid);
}

typedef struct {
    const ora_dg* g;
    const ora_pair* pairs;
    const int64_t* start;
    int W, H, gx, tiles, cadence, tid, nthreads;
    const double* bg;
    double* img;
} ora_dimg_job;

static void* dimg_worker(void* arg)
{
    ora_dimg_job* j = (ora_dimg_job*)arg;
    double T[256], C[256][3];
    for (int t = j->tid; t < j->tiles; t += j->nthreads) {
        int ox = (t % j->gx) * 16, oy = (t / j->gx) * 16;
        for (int p = 0; p < 256; p++) { T[p] = 1.0; C[p][0] = C[p][1] = C[p][2] = 0.0; }
        int64_t s = j->start[t], e = j->start[t + 1], processed = 0;
        for (int64_t k = s; k < e; k++) {
            const ora_dg* g = &j->g[j->pairs[k].gid];
            for (int p = 0; p < 256; p++) {
                double dx = g->px - (double)(ox + p % 16), dy = g->py - (double)(oy + p / 16);
                double power = g->log2o + (-0.5 * ORA_LOG2E * g->con[0]) * dx * dx +
                               (-0.5 * ORA_LOG2E * g->con[2]) * dy * dy + (-ORA_LOG2E * g->con[1]) * dx * dy;
                double w = exp2(power) * T[p];
                for (int ch = 0; ch < 3; ch++) C[p][ch] += g->rgb[ch] * w;
                T[p] -= w;
            }
            processed++;
            if (processed % j->cadence == 0) {
                int sat = 1;
                for (int p = 0; p < 256 && sat; p++) sat = T[p] < 0.0001;
                if (sat) break;
            }
        }
        for (int p = 0; p < 256; p++) {
            int px = ox + p % 16, py = oy + p / 16;
            if (px >= j->W || py >= j->H) continue;
            double* o = j->img + 3 * ((size_t)py * j->W + px);
            double tt = (e - s > 0) ? (T[p] < 0.0001 ? 0.0 : T[p]) : 1.0;
            for (int ch = 0; ch < 3; ch++) o[ch] = (e - s > 0 ? C[p][ch] : 0.0) + tt * j->bg[ch];
        }
    }
    return NULL;
}

/* Per-Gaussian FP64 projection of the float-image path (scene transform,
 * EWA conic, SH colour, tile rectangle), for Gaussians [P0, P1). */
typedef struct {
    const ora_cam* c;
    int P0, P1, W, H, gx, gy;
    double tanx, tany, fx, fy;
    const double *means, *log_scales, *quats, *logits, *shs;
    ora_dg* g;
} ora_dproj_job;

static void* dproj_worker(void* arg)
{
    const ora_dproj_job* j = (const ora_dproj_job*)arg;
    const ora_cam c = *j->c;
    const int W = j->W, H = j->H, gx = j->gx, gy = j->gy;
    const double tanx = j->tanx, tany = j->tany, fx = j->fx, fy = j->fy;
    const double *means = j->means, *log_scales = j->log_scales, *quats = j->quats, *logits = j->logits,
                 *shs = j->shs;
    ora_dg* g = j->g;
    for (int i = j->P0; i < j->P1; i++) {
        /* scene transform in double */
        double o = 1.0 / (1.0 + exp(-logits[i]));
        double s[3], q[4], qn = 0.0;
        for (int k = 0; k < 3; k++) s[k] = exp(log_scales[3 * i + k]);
        for (int k = 0; k < 4; k++) { q[k] = quats[4 * i + k]; qn += q[k] * q[k]; }
        qn = sqrt(qn);
        double r = q[0] / qn, x = q[1] / qn, y = q[2] / qn, z = q[3] / qn;
        double R[3][3] = {{1 - 2 * (y * y + z * z), 2 * (x * y - r * z), 2 * (x * z + r * y)},
                          {2 * (x * y + r * z), 1 - 2 * (x * x + z * z), 2 * (y * z - r * x)},
                          {2 * (x * z - r * y), 2 * (y * z + r * x), 1 - 2 * (x * x + y * y)}};
        double Sg[3][3];
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++) {
                double acc = 0.0;
                for (int k = 0; k < 3; k++) acc += R[a][k] * s[k] * s[k] * R[b][k];
                Sg[a][b] = acc;
            }
        const double* m = means + 3 * i;
        double t[3], hom[4];
        for (int rr = 0; rr < 3; rr++)
            t[rr] = c.view[rr][0] * m[0] + c.view[rr][1] * m[1] + c.view[rr][2] * m[2] + c.view[rr][3];
        if (t[2] <= 0.2) continue;
        for (int rr = 0; rr < 4; rr++)
            hom[rr] = c.proj[rr][0] * m[0] + c.proj[rr][1] * m[1] + c.proj[rr][2] * m[2] + c.proj[rr][3];
        double pw = 1.0 / (hom[3] + 0.0000001);
        double limx = 1.3 * tanx, limy = 1.3 * tany;
        double tz = t[2];
        double tx = fmin(limx, fmax(-limx, t[0] / tz)) * tz, ty = fmin(limy, fmax(-limy, t[1] / tz)) * tz;
        double J[2][3] = {{fx / tz, 0.0, -(fx * tx) / (tz * tz)}, {0.0, fy / tz, -(fy * ty) / (tz * tz)}};
        double Tm[2][3];
        for (int a = 0; a < 2; a++)
            for (int k = 0; k < 3; k++)
                Tm[a][k] = J[a][0] * c.view[0][k] + J[a][1] * c.view[1][k] + J[a][2] * c.view[2][k];
        double cv[2][2];
        for (int a = 0; a < 2; a++)
            for (int b = 0; b < 2; b++) {
                double acc = 0.0;
                for (int k = 0; k < 3; k++)
                    for (int l = 0; l < 3; l++) acc += Tm[a][k] * Sg[k][l] * Tm[b][l];
                cv[a][b] = acc;
            }
        double cxx = cv[0][0] + 0.3, cxy = cv[0][1], cyy = cv[1][1] + 0.3;
        double det = cxx * cyy - cxy * cxy;
        ora_dg* G = &g[i];
        G->con[0] = cyy / det;
        G->con[1] = -cxy / det;
        G->con[2] = cxx / det;
        G->log2o = log2(o);
        double power = ORA_LN2 * 8.0 + ORA_LN2 * G->log2o;
        if (2.0 * det * power < 0.09 * (cxx + cyy) && o < 0.5) continue;
        int w = (int)(1.414214 * sqrt(cxx * power) + 1.0), h = (int)(1.414214 * sqrt(cyy * power) + 1.0);
        G->px = ((hom[0] * pw + 1.0) * W - 1.0) * 0.5;
        G->py = ((hom[1] * pw + 1.0) * H - 1.0) * 0.5;
        G->depth = tz;
        double dir[3] = {m[0] - c.campos[0], m[1] - c.campos[1], m[2] - c.campos[2]};
        double l = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        double X = dir[0] / l, Y = dir[1] / l, Z = dir[2] / l;
        double xx = X * X, yy = Y * Y, zz = Z * Z;
        double B[16] = {C0, -C1 * Y, C1 * Z, -C1 * X, C2[0] * X * Y, C2[1] * Y * Z, C2[2] * (2 * zz - xx - yy),
                        C2[3] * X * Z, C2[4] * (xx - yy), C3[0] * Y * (3 * xx - yy), C3[1] * X * Y * Z,
                        C3[2] * Y * (4 * zz - xx - yy), C3[3] * Z * (2 * zz - 3 * xx - 3 * yy),
                        C3[4] * X * (4 * zz - xx - yy), C3[5] * Z * (xx - yy), C3[6] * X * (xx - 3 * yy)};
        for (int ch = 0; ch < 3; ch++) {
            double acc = 0.5;
            for (int k = 0; k < 16; k++) acc += B[k] * shs[48 * (size_t)i + 3 * k + ch];
            G->rgb[ch] = acc > 0.0 ? acc : 0.0;
        }
        /* tile rectangle as the forward (centre rounded to float) */
        G->power = power;
        double fpx = (float)G->px, fpy = (float)G->py;
        G->x0 = imin(gx, imax(0, (int)((fpx - w) / 16)));
        G->y0 = imin(gy, imax(0, (int)((fpy - h) / 16)));
        G->x1 = imin(gx, imax(0, (int)((fpx + w) / 16) + 1));
        G->y1 = imin(gy, imax(0, (int)((fpy + h) / 16) + 1));
        G->ok = 1;
    }
    return NULL;
}

/* The float image of ora_image_fp64 on the tiles with tile_mask[t] != 0 only
 * (every tile when tile_mask is NULL); the loss sums over those tiles'
 * pixels.  rects_out (optional, [P][4]) receives each Gaussian's tile
 * rectangle x0, y0, x1, y1 (all zero when culled).  A perturbation of one
 * Gaussian changes only the tiles of its rectangle, so finite differences of
 * the loss over those tiles equal those over the whole image. */
double ora_image_fp64_masked(int P, const double* means, const double* log_scales, const double* quats,
                             const double* logits, const double* shs, int W, int H, const float* cam_pos,
                             const float* cam_rot, double fx, double fy, const double* bg, int cadence,
                             const double* target, const uint8_t* tile_mask, int32_t* rects_out, double* img,
                             int nthreads)
{
    ora_cam c;
    make_cam(&c, W, H, cam_pos, cam_rot, fx, fy, 100.0, 0.01);
    const int gx = (W + 15) / 16, gy = (H + 15) / 16, tiles = gx * gy;
    const double tanx = W / (2.0 * fx), tany = H / (2.0 * fy);
    ora_dg* g = (ora_dg*)calloc((size_t)(P > 0 ? P : 1), sizeof(ora_dg));
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    {
        pthread_t pth[256];
        ora_dproj_job pj[256];
        const int per = (P + nthreads - 1) / nthreads;
        for (int t = 0; t < nthreads; t++) {
            ora_dproj_job* jb = &pj[t];
            jb->c = &c; jb->W = W; jb->H = H; jb->gx = gx; jb->gy = gy;
            jb->tanx = tanx; jb->tany = tany; jb->fx = fx; jb->fy = fy;
            jb->means = means; jb->log_scales = log_scales; jb->quats = quats; jb->logits = logits; jb->shs = shs;
            jb->g = g;
            jb->P0 = imin(P, t * per);
            jb->P1 = imin(P, (t + 1) * per);
        }
        for (int t = 1; t < nthreads; t++) pthread_create(&pth[t], NULL, dproj_worker, &pj[t]);
        dproj_worker(&pj[0]);
        for (int t = 1; t < nthreads; t++) pthread_join(pth[t], NULL);
    }
    int64_t cap = 1024, n = 0;
    ora_pair* pairs = (ora_pair*)malloc(sizeof(ora_pair) * cap);
    for (int i = 0; i < P; i++) {
        const ora_dg* G = &g[i];
        if (rects_out) {
            rects_out[4 * (size_t)i + 0] = G->ok ? G->x0 : 0;
            rects_out[4 * (size_t)i + 1] = G->ok ? G->y0 : 0;
            rects_out[4 * (size_t)i + 2] = G->ok ? G->x1 : 0;
            rects_out[4 * (size_t)i + 3] = G->ok ? G->y1 : 0;
        }
        if (!G->ok) continue;
        ora_geom tg;
        memset(&tg, 0, sizeof tg);
        tg.px = G->px; tg.py = G->py; tg.power = G->power;
        tg.con[0] = G->con[0]; tg.con[1] = G->con[1]; tg.con[2] = G->con[2];
        for (int yy2 = G->y0; yy2 < G->y1; yy2++)
            for (int xx2 = G->x0; xx2 < G->x1; xx2++) {
                const int t = yy2 * gx + xx2;
                if (tile_mask && !tile_mask[t]) continue;
                if (!tile_hit(&tg, xx2, yy2, 16, 16)) continue;
                if (n == cap) { cap *= 2; pairs = (ora_pair*)realloc(pairs, sizeof(ora_pair) * cap); }
                pairs[n].tile = (uint32_t)t;
                pairs[n].depth = G->depth;
                pairs[n].gid = (uint32_t)i;
                n++;
            }
    }
    qsort(pairs, (size_t)n, sizeof(ora_pair), pair_cmp);
    int64_t* start = (int64_t*)calloc((size_t)tiles + 1, sizeof(int64_t));
    for (int64_t k = 0; k < n; k++) start[pairs[k].tile + 1]++;
    for (int t = 0; t < tiles; t++) start[t + 1] += start[t];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    ora_dimg_job jobs[256];
    for (int i = 0; i < nthreads; i++) {
        ora_dimg_job* jb = &jobs[i];
        jb->g = g; jb->pairs = pairs; jb->start = start; jb->W = W; jb->H = H; jb->gx = gx; jb->tiles = tiles;
        jb->cadence = cadence > 0 ? cadence : 1; jb->tid = i; jb->nthreads = nthreads; jb->bg = bg; jb->img = img;
    }
    for (int i = 1; i < nthreads; i++) pthread_create(&th[i], NULL, dimg_worker, &jobs[i]);
    dimg_worker(&jobs[0]);
    for (int i = 1; i < nthreads; i++) pthread_join(th[i], NULL);
    double loss = 0.0;
    if (target)
        for (size_t k = 0; k < (size_t)W * H * 3; k++) {
            if (tile_mask) {
                const size_t px = k / 3;
                if (!tile_mask[((int)(px / W) / 16) * gx + (int)(px % W) / 16]) continue;
            }
            double d = img[k] - target[k];
            loss += d * d;
        }
    free(start);
    free(pairs);
    free(g);
    return loss;
}

double ora_image_fp64(int P, const double* means, const double* log_scales, const double* quats,
                      const double* logits, const double* shs, int W, int H, const float* cam_pos,
                      const float* cam_rot, double fx, double fy, const double* bg, int cadence,
                      const double* target, double* img, int nthreads)
{
    return ora_image_fp64_masked(P, means, log_scales, quats, logits, shs, W, H, cam_pos, cam_rot, fx, fy, bg,
                                 cadence, target, NULL, NULL, img, nthreads);
}
