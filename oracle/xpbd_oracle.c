/*
 * CPU oracle for the XPBD particle substep — TEST INFRASTRUCTURE ONLY.
 * See xpbd_oracle.h for scope, canonical orders and parity status.
 *
 * Every function below cites the reference file:line it restates. Arithmetic
 * is written operation by operation in the order GLSL evaluates it; explicit
 * fma() calls appear exactly where the shaders write fma(); the file is built
 * with -ffp-contract=off so that nothing else is fused.
 */
#include "xpbd_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifdef OR_F64
typedef double real;
#define RF(x) x
#define R_FMA fma
#define R_SQRT sqrt
#define R_FLOOR floor
#define R_FABS fabs
#else
typedef float real;
#define RF(x) x##f
#define R_FMA fmaf
#define R_SQRT sqrtf
#define R_FLOOR floorf
#define R_FABS fabsf
#endif

int or_precision(void) {
#ifdef OR_F64
    return 2;
#else
    return 1;
#endif
}

static int g_threads = 0;
void or_set_threads(int n) { g_threads = n; }
int or_get_threads(void) {
#ifdef _OPENMP
    return g_threads > 0 ? g_threads : omp_get_max_threads();
#else
    return 1;
#endif
}
#ifdef _OPENMP
#define OMP_THREADS num_threads(or_get_threads())
#endif

/* ------------------------------------------------------------------------- */
/* GLSL built-ins with a fixed evaluation order                               */
/* ------------------------------------------------------------------------- */
typedef struct { real x, y, z; } v3;
static inline v3 mk(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 vmuls(v3 a, real s) { return mk(a.x * s, a.y * s, a.z * s); }
static inline v3 vneg(v3 a) { return mk(-a.x, -a.y, -a.z); }
/* GLSL max(x,y): y if x < y else x; min(x,y): y if y < x else x */
static inline real gmax(real a, real b) { return a < b ? b : a; }
static inline real gmin(real a, real b) { return b < a ? b : a; }
static inline real gclamp(real x, real lo, real hi) { return gmin(gmax(x, lo), hi); }
/* dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z */
static inline real vdot(v3 a, v3 b) { return (a.x * b.x + a.y * b.y) + a.z * b.z; }
static inline v3 vcross(v3 a, v3 b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static inline real vlength(v3 a) { return R_SQRT(vdot(a, a)); }
/* normalize(v) = v / length(v), component-wise IEEE division */
static inline v3 vnormalize(v3 a) {
    real l = vlength(a);
    return mk(a.x / l, a.y / l, a.z / l);
}
static inline v3 vfma_vs(v3 a, real s, v3 c) { /* fma(a, vec3(s), c) */
    return mk(R_FMA(a.x, s, c.x), R_FMA(a.y, s, c.y), R_FMA(a.z, s, c.z));
}

/* exact_sqrt: solve_particle_particle_contacts.comp:81-85 (same in the shape/mesh shaders).
 * At a == 0 the refinement evaluates fma(0, 0.5 / 0, 0), NaN in IEEE arithmetic and
 * undefined under Vulkan's division rules; the refinement is meant to equal sqrt(a),
 * so a is returned (a particle lying exactly on a mesh surface keeps a finite contact). */
static inline real exact_sqrt(real a) {
    if (a == RF(0.0)) return a;
    real d = R_SQRT(a);
    real r = R_FMA(-d, d, a);
    return R_FMA(r, RF(0.5) / d, d);
}
/* exact_length: solve_particle_particle_contacts.comp:87-92 */
static inline real exact_length(v3 a) {
    real yy = a.y * a.y;
    real xx_yy = R_FMA(a.x, a.x, yy);
    real sq = R_FMA(a.z, a.z, xx_yy);
    return exact_sqrt(sq);
}
/* exact_dot: solve_particle_particle_contacts.comp:94-98 (= exact_dot3, generate_mesh_contacts.comp:64-68) */
static inline real exact_dot(v3 a, v3 b) {
    real y = a.y * b.y;
    real x_y = R_FMA(a.x, b.x, y);
    return R_FMA(a.z, b.z, x_y);
}
/* exact_div: solve_particle_particle_contacts.comp:100-105 (shape/mesh shaders identical) */
static inline v3 exact_div(v3 v, real d) {
    real inv_d = RF(1.0) / d;
    v3 q = vmuls(v, inv_d);
    v3 rem = mk(R_FMA(-d, q.x, v.x), R_FMA(-d, q.y, v.y), R_FMA(-d, q.z, v.z));
    return mk(R_FMA(rem.x, inv_d, q.x), R_FMA(rem.y, inv_d, q.y), R_FMA(rem.z, inv_d, q.z));
}
/* exact_div1: generate_mesh_contacts.comp:57-62 */
static inline real exact_div1(real v, real d) {
    real inv_d = RF(1.0) / d;
    real q = v * inv_d;
    real rem = R_FMA(-d, q, v);
    return R_FMA(rem, inv_d, q);
}
/* exact_div of apply_particle_deltas.comp:30-36 (Markstein form) */
static inline v3 exact_div_apply(v3 a, real b) {
    real y = RF(1.0) / b;
    y = R_FMA(-b, y, RF(1.0)) * y + y;
    v3 q = vmuls(a, y);
    v3 r = mk(R_FMA(-q.x, b, a.x), R_FMA(-q.y, b, a.y), R_FMA(-q.z, b, a.z));
    return mk(R_FMA(r.x, y, q.x), R_FMA(r.y, y, q.y), R_FMA(r.z, y, q.z));
}
/* diff_product: generate_mesh_contacts.comp:70-75 */
static inline real diff_product(real a, real b, real c, real d) {
    real cd = c * d;
    real diff = R_FMA(a, b, -cd);
    real err = R_FMA(-c, d, cd);
    return diff + err;
}

/*
 * acos(x), x in [-1,1]. GLSL leaves acos's rounding to the GPU driver; this code
 * fixes it to a Taylor series of asin (coefficients (2n)!/(4^n (n!)^2 (2n+1)),
 * n=1..11, rounded to float) evaluated by Horner in t^2, with the half-angle
 * identity acos(x) = 2 asin(sqrt((1-x)/2)) for |x| > 1/2. Max error ~1 ulp.
 * The CUDA kernels evaluate the identical expression, so both agree bit for bit.
 */
static float asin_series_f(float t) {
    static const float c[11] = {
        0x1.555556p-3f, 0x1.333334p-4f, 0x1.6db6dcp-5f, 0x1.f1c71cp-6f, 0x1.6e8ba2p-6f,
        0x1.1c4ec4p-6f, 0x1.c9999ap-7f, 0x1.7a8788p-7f, 0x1.3fde50p-7f, 0x1.12ef3cp-7f,
        0x1.df3bd4p-8f};
    float t2 = t * t;
    float acc = c[10];
    for (int k = 9; k >= 0; k--) acc = acc * t2 + c[k];
    acc = acc * t2;
    return t + t * acc;
}
float or_acos(float x) {
    const float half_pi = 0x1.921fb6p+0f;
    const float pi = 0x1.921fb6p+1f;
    float ax = fabsf(x);
    if (ax <= 0.5f) return half_pi - asin_series_f(x);
    float s = sqrtf((1.0f - ax) * 0.5f);
    float a = 2.0f * asin_series_f(s);
    return x > 0.0f ? a : pi - a;
}
static inline real r_acos(real x) {
#ifdef OR_F64
    return acos(x);
#else
    return or_acos(x);
#endif
}

/* float -> int conversion of an integral float, saturating; NaN -> 0.
 * (GLSL int() of out-of-range values is undefined; the kernels use the same rule.) */
static inline int32_t f2i(real f) {
    if (!(f == f)) return 0;
    if (f >= RF(1073741824.0)) return 1073741824;
    if (f <= RF(-1073741824.0)) return -1073741824;
    return (int32_t)f;
}

/* quat_rotate / quat_rotate_inv: solve_particle_shape_contacts.comp:50-68 */
typedef struct { real x, y, z, w; } q4;
static inline v3 quat_rotate(q4 q, v3 x) {
    real c = RF(2.0) * q.w * q.w - RF(1.0);
    real d = RF(2.0) * ((q.x * x.x + q.y * x.y) + q.z * x.z);
    return mk((x.x * c + q.x * d) + (q.y * x.z - q.z * x.y) * q.w * RF(2.0),
              (x.y * c + q.y * d) + (q.z * x.x - q.x * x.z) * q.w * RF(2.0),
              (x.z * c + q.z * d) + (q.x * x.y - q.y * x.x) * q.w * RF(2.0));
}
static inline v3 quat_rotate_inv(q4 q, v3 x) {
    real c = RF(2.0) * q.w * q.w - RF(1.0);
    real d = RF(2.0) * ((q.x * x.x + q.y * x.y) + q.z * x.z);
    return mk((x.x * c + q.x * d) - (q.y * x.z - q.z * x.y) * q.w * RF(2.0),
              (x.y * c + q.y * d) - (q.z * x.x - q.x * x.z) * q.w * RF(2.0),
              (x.z * c + q.z * d) - (q.x * x.y - q.y * x.x) * q.w * RF(2.0));
}

/* ------------------------------------------------------------------------- */
/* Scene state                                                                 */
/* ------------------------------------------------------------------------- */
#define GRID_DIM 128
#define NUM_CELLS (GRID_DIM * GRID_DIM * GRID_DIM)

typedef struct {
    float* verts;
    int64_t nv;
    uint32_t* tris;
    int64_t nt;
    float margin;
    float rot[4];
    int watertight;
    /* per-mesh BVH as built (local indices), 4 floats per node half */
    float* lowers;
    float* uppers;
    uint32_t* prims;
    uint32_t root;
    int64_t n_nodes;
    float avg_edge;
} or_mesh;

/* Stored trajectory of a differentiable rollout. */
typedef struct {
    int64_t steps;      /* substeps stored */
    real *x, *v;        /* (steps + 1) x 3n: state at the start of every substep, then the final */
    real sdt, inv;
    int clamped;
} or_traj;

/* Rigid contact generated for one vertex of a dynamic body's mesh (shape0 = that
 * body's mesh shape): the record solve_body_contact_positions.comp:8-18 reads. */
#define RC_CAP 4 /* contacts per vertex */
typedef struct {
    int32_t shape1;   /* 0 = ground plane, m + 1 = mesh m */
    v3 p0, p1;        /* contact points in the frames of shape0's and shape1's bodies */
    v3 off0, off1;    /* surface offsets in the same frames */
    v3 n;             /* world normal, pointing from shape0 to shape1 */
    real th0, th1;    /* thicknesses (shape margins) */
} or_rcontact;

struct or_solver {
    or_config cfg;
    int64_t n, cmax;
    real *x, *v, *x0, *v0, *xo, *vo, *w, *r, *delta, *vsnap;
    int32_t* flags;
    /* contacts (SoA, canonical slot order) */
    int64_t ccount_raw;
    int32_t *cpart, *cshape;
    real *cbpos, *cbvel, *cnorm;
    /* hash grid */
    uint32_t *cells, *ids, *scells, *sids;
    int32_t *cstart, *cend;
    /* meshes */
    int64_t nmesh, mesh_cap;
    or_mesh* meshes;
    int finalized;
    float* all_verts;
    float* all_vels;
    int64_t n_all_verts;
    uint32_t* all_tris;
    int64_t n_all_tris;
    float *nl, *nu; /* packed global node halves, 4 floats each */
    int64_t total_nodes;
    uint32_t* prim;
    int64_t total_prims;
    uint32_t* roots;
    uint32_t *prim_off, *prim_cnt;
    /* shapes and bodies: shape 0 = plane (body -1), shape c+1 = mesh c (body c) */
    int32_t* shape_body;
    real* shape_mu;
    int64_t nbody;
    real *body_q, *body_qd, *body_com, *body_invI, *body_invm;
    int32_t* body_flags;
    /* dynamic bodies (extension): inertia, substep-start and mid-iteration states */
    real *body_I, *body_qp, *body_qdp, *body_qm, *body_qdm;
    int dyn_any;
    or_body_params bp;
    real* bdel;       /* per contact slot: body delta (lin xyz, ang xyz) */
    uint8_t* bvalid;  /* per contact slot: bdel holds a contribution */
    int32_t* rc_cnt;  /* per vertex of the concatenated vertex array */
    or_rcontact* rc;  /* RC_CAP per vertex */
    int64_t rc_overflow, partner_dummy;
    or_traj traj;     /* differentiable rollout */
};

static void* xcalloc(size_t n, size_t sz) {
    void* p = calloc(n ? n : 1, sz);
    if (!p) {
        fprintf(stderr, "oracle: out of memory\n");
        abort();
    }
    return p;
}

or_solver* or_create(const or_config* cfg, int64_t n, int64_t max_contacts) {
    or_solver* s = (or_solver*)xcalloc(1, sizeof(or_solver));
    s->cfg = *cfg;
    s->n = n;
    s->cmax = max_contacts ? max_contacts : n * 2; /* scene.cpp:68 */
    size_t n3 = (size_t)n * 3;
    s->x = xcalloc(n3, sizeof(real));
    s->v = xcalloc(n3, sizeof(real));
    s->x0 = xcalloc(n3, sizeof(real));
    s->v0 = xcalloc(n3, sizeof(real));
    s->xo = xcalloc(n3, sizeof(real));
    s->vo = xcalloc(n3, sizeof(real));
    s->delta = xcalloc(n3, sizeof(real));
    s->vsnap = xcalloc(n3, sizeof(real));
    s->w = xcalloc((size_t)n, sizeof(real));
    s->r = xcalloc((size_t)n, sizeof(real));
    s->flags = xcalloc((size_t)n, sizeof(int32_t));
    s->cpart = xcalloc((size_t)s->cmax, sizeof(int32_t));
    s->cshape = xcalloc((size_t)s->cmax, sizeof(int32_t));
    s->cbpos = xcalloc((size_t)s->cmax * 3, sizeof(real));
    s->cbvel = xcalloc((size_t)s->cmax * 3, sizeof(real));
    s->cnorm = xcalloc((size_t)s->cmax * 3, sizeof(real));
    s->bdel = xcalloc((size_t)s->cmax * 6, sizeof(real));
    s->bvalid = xcalloc((size_t)s->cmax, sizeof(uint8_t));
    s->bp.angular_damping = 0.0f;
    s->bp.rigid_contact_margin = 0.01f;
    s->bp.rigid_contact_relaxation = 0.8f;
    s->bp.rigid_contact_con_weighting = 1;
    s->bp.rigid_mu_torsional = 0.0f;
    s->bp.rigid_mu_rolling = 0.0f;
    s->bp.particle_contact_con_weighting = 1;
    s->cells = xcalloc((size_t)n, sizeof(uint32_t));
    s->ids = xcalloc((size_t)n, sizeof(uint32_t));
    s->scells = xcalloc((size_t)n, sizeof(uint32_t));
    s->sids = xcalloc((size_t)n, sizeof(uint32_t));
    s->cstart = xcalloc(NUM_CELLS, sizeof(int32_t));
    s->cend = xcalloc(NUM_CELLS, sizeof(int32_t));
    s->mesh_cap = 4;
    s->meshes = xcalloc((size_t)s->mesh_cap, sizeof(or_mesh));
    return s;
}

static void free_finalized(or_solver* s) {
    free(s->all_verts); free(s->all_vels); free(s->all_tris); free(s->nl); free(s->nu);
    free(s->prim); free(s->roots); free(s->prim_off); free(s->prim_cnt);
    free(s->shape_body); free(s->shape_mu);
    free(s->body_q); free(s->body_qd); free(s->body_com); free(s->body_invI); free(s->body_invm);
    free(s->body_flags);
    free(s->body_I); free(s->body_qp); free(s->body_qdp); free(s->body_qm); free(s->body_qdm);
    free(s->rc_cnt); free(s->rc);
    s->body_I = s->body_qp = s->body_qdp = s->body_qm = s->body_qdm = NULL;
    s->rc_cnt = NULL;
    s->rc = NULL;
    s->dyn_any = 0;
    s->all_verts = s->all_vels = NULL; s->all_tris = NULL; s->nl = s->nu = NULL; s->prim = NULL;
    s->roots = s->prim_off = s->prim_cnt = NULL; s->shape_body = NULL; s->shape_mu = NULL;
    s->body_q = s->body_qd = s->body_com = s->body_invI = s->body_invm = NULL; s->body_flags = NULL;
}

void or_destroy(or_solver* s) {
    if (!s) return;
    free(s->x); free(s->v); free(s->x0); free(s->v0); free(s->xo); free(s->vo); free(s->delta);
    free(s->vsnap); free(s->w); free(s->r); free(s->flags);
    free(s->cpart); free(s->cshape); free(s->cbpos); free(s->cbvel); free(s->cnorm);
    free(s->bdel); free(s->bvalid);
    free(s->traj.x); free(s->traj.v);
    free(s->cells); free(s->ids); free(s->scells); free(s->sids); free(s->cstart); free(s->cend);
    for (int64_t m = 0; m < s->nmesh; m++) {
        free(s->meshes[m].verts); free(s->meshes[m].tris); free(s->meshes[m].lowers);
        free(s->meshes[m].uppers); free(s->meshes[m].prims);
    }
    free(s->meshes);
    free_finalized(s);
    free(s);
}

/* ------------------------------------------------------------------------- */
/* Mesh helpers: watertight test (scene.cpp:170-198), LBVH (mesh_lbvh.h:49-223) */
/* ------------------------------------------------------------------------- */
static int cmp_edge(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}
int or_tris_watertight(const uint32_t* tris, int64_t nt, int64_t nv) {
    if (nt == 0 || nv == 0) return 0;
    uint64_t* e = xcalloc((size_t)nt * 3, sizeof(uint64_t));
    for (int64_t t = 0; t < nt; t++) {
        for (int k = 0; k < 3; k++) {
            uint32_t a = tris[t * 3 + k], b = tris[t * 3 + (k + 1) % 3];
            uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
            e[t * 3 + k] = ((uint64_t)lo << 32) | hi;
        }
    }
    qsort(e, (size_t)nt * 3, sizeof(uint64_t), cmp_edge);
    int closed = 1;
    size_t i = 0, m = (size_t)nt * 3;
    while (i < m) {
        size_t j = i + 1;
        while (j < m && e[j] == e[i]) j++;
        if (j - i != 2) { closed = 0; break; }
        i = j;
    }
    free(e);
    return closed;
}

static uint32_t part1by2(uint32_t n) { /* mesh_lbvh.h:12-19 */
    n &= 0x000003ffu;
    n = (n ^ (n << 16)) & 0xff0000ffu;
    n = (n ^ (n << 8)) & 0x0300f00fu;
    n = (n ^ (n << 4)) & 0x030c30c3u;
    n = (n ^ (n << 2)) & 0x09249249u;
    return n;
}
static uint32_t morton3_1024(float x, float y, float z) { /* mesh_lbvh.h:21-29 */
    int ix = (int)(x * 1024.0f), iy = (int)(y * 1024.0f), iz = (int)(z * 1024.0f);
    uint32_t ux = (uint32_t)(ix < 0 ? 0 : (ix > 1023 ? 1023 : ix));
    uint32_t uy = (uint32_t)(iy < 0 ? 0 : (iy > 1023 ? 1023 : iy));
    uint32_t uz = (uint32_t)(iz < 0 ? 0 : (iz > 1023 ? 1023 : iz));
    return (part1by2(uz) << 2) | (part1by2(uy) << 1) | part1by2(ux);
}
static inline float fminr(float a, float b) { return b < a ? b : a; } /* std::min */
static inline float fmaxr(float a, float b) { return a < b ? b : a; } /* std::max */
static inline uint32_t f2u(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float u2f(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }

/* lowers/uppers: 2*ntris nodes x 4 floats, w = packed uint32 bits */
int or_bvh_build(const float* pts, int64_t num_pts, const uint32_t* tris, int64_t num_tris,
                 float* lowers, float* uppers, uint32_t* prims, uint32_t* root_out) {
    (void)num_pts;
    const uint32_t n = (uint32_t)num_tris;
    if (n == 0) return -1;
    float* blo = xcalloc((size_t)n * 3, sizeof(float));
    float* bhi = xcalloc((size_t)n * 3, sizeof(float));
    float tlo[3] = {1e30f, 1e30f, 1e30f}, thi[3] = {-1e30f, -1e30f, -1e30f};
    for (uint32_t t = 0; t < n; t++) {
        for (int a = 0; a < 3; a++) blo[t * 3 + a] = bhi[t * 3 + a] = pts[tris[t * 3 + 0] * 3 + a];
        for (int k = 1; k < 3; k++) {
            const float* p = &pts[tris[t * 3 + k] * 3];
            for (int a = 0; a < 3; a++) {
                blo[t * 3 + a] = fminr(blo[t * 3 + a], p[a]);
                bhi[t * 3 + a] = fmaxr(bhi[t * 3 + a], p[a]);
            }
        }
        for (int a = 0; a < 3; a++) {
            tlo[a] = fminr(tlo[a], blo[t * 3 + a]);
            thi[a] = fmaxr(thi[a], bhi[t * 3 + a]);
        }
    }
    float inv_e[3];
    for (int a = 0; a < 3; a++) inv_e[a] = 1.0f / ((thi[a] - tlo[a]) + 0.0001f);
    uint32_t* key = xcalloc(n, sizeof(uint32_t));
    uint32_t* idx = xcalloc(n, sizeof(uint32_t));
    for (uint32_t t = 0; t < n; t++) {
        float loc[3];
        for (int a = 0; a < 3; a++) {
            float c = 0.5f * (blo[t * 3 + a] + bhi[t * 3 + a]);
            loc[a] = (c - tlo[a]) * inv_e[a];
        }
        key[t] = morton3_1024(loc[0], loc[1], loc[2]);
        idx[t] = t;
    }
    /* stable sort by key (std::stable_sort): LSD radix, 4 x 8 bits */
    {
        uint32_t* k2 = xcalloc(n, sizeof(uint32_t));
        uint32_t* i2 = xcalloc(n, sizeof(uint32_t));
        for (int pass = 0; pass < 4; pass++) {
            uint32_t cnt[257] = {0};
            int sh = pass * 8;
            for (uint32_t t = 0; t < n; t++) cnt[((key[t] >> sh) & 255u) + 1]++;
            for (int b = 0; b < 256; b++) cnt[b + 1] += cnt[b];
            for (uint32_t t = 0; t < n; t++) {
                uint32_t d = (key[t] >> sh) & 255u;
                k2[cnt[d]] = key[t];
                i2[cnt[d]] = idx[t];
                cnt[d]++;
            }
            uint32_t* tk = key; key = k2; k2 = tk;
            uint32_t* ti = idx; idx = i2; i2 = ti;
        }
        free(k2); free(i2);
    }
    for (uint32_t t = 0; t < n; t++) prims[t] = idx[t];
    int* deltas = xcalloc(n > 1 ? n - 1 : 1, sizeof(int));
    for (uint32_t i = 0; i + 1 < n; i++) {
        uint64_t xo = (uint64_t)key[i] ^ (uint64_t)key[i + 1];
        deltas[i] = xo == 0 ? 64 : __builtin_clzll(xo);
    }
    const uint32_t max_nodes = 2 * n;
    memset(lowers, 0, sizeof(float) * 4 * max_nodes);
    memset(uppers, 0, sizeof(float) * 4 * max_nodes);
    uint32_t* lp = xcalloc(max_nodes, sizeof(uint32_t)); /* packed words */
    uint32_t* up = xcalloc(max_nodes, sizeof(uint32_t));
    int* parents = xcalloc(max_nodes, sizeof(int));
    int* nchild = xcalloc(max_nodes, sizeof(int));
    int* rl = xcalloc(max_nodes, sizeof(int));
    int* rr = xcalloc(max_nodes, sizeof(int));
    for (uint32_t i = 0; i < max_nodes; i++) parents[i] = -1;
    for (uint32_t i = 0; i < n; i++) {
        uint32_t it = prims[i];
        for (int a = 0; a < 3; a++) {
            lowers[i * 4 + a] = blo[it * 3 + a];
            uppers[i * 4 + a] = bhi[it * 3 + a];
        }
        lp[i] = i | (1u << 30);
        up[i] = i + 1;
        rl[i] = (int)i;
        rr[i] = (int)i;
    }
    uint32_t root = 0;
    const int off = (int)n;
    for (uint32_t i = 0; i < n; i++) { /* bottom-up parent selection, mesh_lbvh.h:148-203 */
        int curr = (int)i;
        for (;;) {
            int left = rl[curr], right = rr[curr];
            if (left == 0 && right == (int)(n - 1)) {
                root = (uint32_t)curr;
                parents[curr] = -1;
                break;
            }
            int parent_right;
            if (left == 0) {
                parent_right = 1;
            } else if (right != (int)(n - 1) && deltas[right] >= deltas[left - 1]) {
                if (deltas[right] == deltas[left - 1])
                    parent_right = (int)((prims[left - 1] % 2) ^ (prims[right] % 2));
                else
                    parent_right = 1;
            } else {
                parent_right = 0;
            }
            int parent;
            if (parent_right) {
                parent = right + off;
                parents[curr] = parent;
                lp[parent] = (uint32_t)curr;
                rl[parent] = left;
            } else {
                parent = left + off - 1;
                parents[curr] = parent;
                up[parent] = (uint32_t)curr;
                rr[parent] = right;
            }
            nchild[parent]++;
            if (nchild[parent] == 1) break;
            int lc = (int)(lp[parent] & 0x3FFFFFFFu), rc = (int)(up[parent] & 0x3FFFFFFFu);
            for (int a = 0; a < 3; a++) {
                lowers[parent * 4 + a] = fminr(lowers[lc * 4 + a], lowers[rc * 4 + a]);
                uppers[parent * 4 + a] = fmaxr(uppers[lc * 4 + a], uppers[rc * 4 + a]);
            }
            curr = parent;
        }
    }
    for (uint32_t ni = 0; ni < max_nodes; ni++) { /* mark_packed_leaf_nodes, mesh_lbvh.h:205-222 */
        if (nchild[ni] > 0 || ni < n) {
            int depth = 1;
            int p = parents[ni];
            while (p != -1) {
                p = parents[p];
                depth++;
            }
            int left = rl[ni], right = rr[ni] + 1;
            if (right - left <= 4 || depth >= 32) {
                lp[ni] = (uint32_t)left | (1u << 30);
                up[ni] = (uint32_t)right;
            }
        }
    }
    for (uint32_t ni = 0; ni < max_nodes; ni++) {
        lowers[ni * 4 + 3] = u2f(lp[ni]);
        uppers[ni * 4 + 3] = u2f(up[ni]);
    }
    *root_out = root;
    free(blo); free(bhi); free(key); free(idx); free(deltas); free(lp); free(up); free(parents);
    free(nchild); free(rl); free(rr);
    return 0;
}

/* MeshBvh::refit_recursive (mesh_bvh.h:142-175), iterative post-order */
static void refit_node(const float* pts, const uint32_t* tris, float* lo4, float* hi4,
                       const uint32_t* prims, uint32_t ni) {
    uint32_t lpk = f2u(lo4[ni * 4 + 3]);
    if ((lpk >> 30) & 3u) {
        uint32_t a0 = lpk & 0x3FFFFFFFu, a1 = f2u(hi4[ni * 4 + 3]) & 0x3FFFFFFFu;
        float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f};
        for (uint32_t pi = a0; pi < a1; pi++) {
            uint32_t t = prims[pi];
            for (int k = 0; k < 3; k++) {
                uint32_t idx = tris[t * 3 + k];
                for (int a = 0; a < 3; a++) {
                    lo[a] = fminr(lo[a], pts[idx * 3 + a]);
                    hi[a] = fmaxr(hi[a], pts[idx * 3 + a]);
                }
            }
        }
        for (int a = 0; a < 3; a++) { lo4[ni * 4 + a] = lo[a]; hi4[ni * 4 + a] = hi[a]; }
    } else {
        uint32_t l = lpk & 0x3FFFFFFFu, r = f2u(hi4[ni * 4 + 3]);
        refit_node(pts, tris, lo4, hi4, prims, l);
        refit_node(pts, tris, lo4, hi4, prims, r);
        for (int a = 0; a < 3; a++) {
            lo4[ni * 4 + a] = fminr(lo4[l * 4 + a], lo4[r * 4 + a]);
            hi4[ni * 4 + a] = fmaxr(hi4[l * 4 + a], hi4[r * 4 + a]);
        }
    }
}
void or_bvh_refit(const float* pts, const uint32_t* tris, float* lowers, float* uppers,
                  const uint32_t* prims, uint32_t root) {
    refit_node(pts, tris, lowers, uppers, prims, root);
}

/* ------------------------------------------------------------------------- */
/* Scene construction                                                          */
/* ------------------------------------------------------------------------- */
int or_add_mesh(or_solver* s, const float* verts, int64_t nv, const uint32_t* tris, int64_t nt,
                float margin, const float* rot, int wt_override) { /* scene.cpp:154-202 */
    if (s->nmesh == s->mesh_cap) {
        s->mesh_cap *= 2;
        s->meshes = realloc(s->meshes, sizeof(or_mesh) * (size_t)s->mesh_cap);
    }
    or_mesh* m = &s->meshes[s->nmesh++];
    memset(m, 0, sizeof(*m));
    m->verts = xcalloc((size_t)nv * 3, sizeof(float));
    memcpy(m->verts, verts, sizeof(float) * 3 * (size_t)nv);
    m->tris = xcalloc((size_t)nt * 3, sizeof(uint32_t));
    memcpy(m->tris, tris, sizeof(uint32_t) * 3 * (size_t)nt);
    m->nv = nv;
    m->nt = nt;
    m->margin = margin;
    m->rot[0] = m->rot[1] = m->rot[2] = 0.0f;
    m->rot[3] = 1.0f;
    if (rot) memcpy(m->rot, rot, sizeof(float) * 4);
    m->watertight = wt_override >= 0 ? (wt_override != 0) : or_tris_watertight(tris, nt, nv);
    s->finalized = 0;
    return 0;
}

int or_finalize_meshes(or_solver* s) { /* scene.cpp:204-390 */
    free_finalized(s);
    int64_t nm = s->nmesh, nshapes = 1 + nm;
    s->shape_body = xcalloc((size_t)nshapes, sizeof(int32_t));
    s->shape_mu = xcalloc((size_t)nshapes, sizeof(real));
    s->shape_body[0] = -1;
    for (int64_t c = 0; c < nm; c++) s->shape_body[1 + c] = (int32_t)c;
    for (int64_t i = 0; i < nshapes; i++) s->shape_mu[i] = (real)s->cfg.shape_material_mu;
    s->nbody = nm;
    s->body_q = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    s->body_qd = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    s->body_com = xcalloc((size_t)(nm ? nm : 1) * 3, sizeof(real));
    s->body_invI = xcalloc((size_t)(nm ? nm : 1) * 9, sizeof(real));
    s->body_invm = xcalloc((size_t)(nm ? nm : 1), sizeof(real));
    s->body_flags = xcalloc((size_t)(nm ? nm : 1), sizeof(int32_t));
    s->body_I = xcalloc((size_t)(nm ? nm : 1) * 9, sizeof(real));
    s->body_qp = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    s->body_qdp = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    s->body_qm = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    s->body_qdm = xcalloc((size_t)(nm ? nm : 1) * 8, sizeof(real));
    for (int64_t b = 0; b < nm; b++) s->body_q[b * 8 + 7] = RF(1.0);

    int64_t tv = 0, tt = 0;
    for (int64_t c = 0; c < nm; c++) { tv += s->meshes[c].nv; tt += s->meshes[c].nt; }
    s->n_all_verts = tv;
    s->n_all_tris = tt;
    s->rc_cnt = xcalloc((size_t)(tv ? tv : 1), sizeof(int32_t));
    s->rc = xcalloc((size_t)(tv ? tv : 1) * RC_CAP, sizeof(or_rcontact));
    s->all_verts = xcalloc((size_t)tv * 3, sizeof(float));
    s->all_vels = xcalloc((size_t)tv * 3, sizeof(float));
    s->all_tris = xcalloc((size_t)tt * 3, sizeof(uint32_t));
    int64_t total_nodes = 0, total_prims = 0;
    for (int64_t c = 0, vo = 0, to = 0; c < nm; c++) {
        or_mesh* m = &s->meshes[c];
        memcpy(s->all_verts + vo * 3, m->verts, sizeof(float) * 3 * (size_t)m->nv);
        for (int64_t k = 0; k < m->nt * 3; k++) s->all_tris[to * 3 + k] = m->tris[k] + (uint32_t)vo;
        free(m->lowers); free(m->uppers); free(m->prims);
        m->n_nodes = 2 * m->nt;
        m->lowers = xcalloc((size_t)m->n_nodes * 4, sizeof(float));
        m->uppers = xcalloc((size_t)m->n_nodes * 4, sizeof(float));
        m->prims = xcalloc((size_t)m->nt, sizeof(uint32_t));
        /* the build sees the concatenated vertex array with rebased indices (scene.cpp:263-270) */
        or_bvh_build(s->all_verts, vo + m->nv, s->all_tris + to * 3, m->nt, m->lowers, m->uppers,
                     m->prims, &m->root);
        double sum_len = 0.0; /* scene.cpp:274-281 */
        for (int64_t t = 0; t < m->nt; t++) {
            for (int e = 0; e < 3; e++) {
                uint32_t i0 = s->all_tris[(to + t) * 3 + e], i1 = s->all_tris[(to + t) * 3 + (e + 1) % 3];
                float dx = s->all_verts[i1 * 3] - s->all_verts[i0 * 3];
                float dy = s->all_verts[i1 * 3 + 1] - s->all_verts[i0 * 3 + 1];
                float dz = s->all_verts[i1 * 3 + 2] - s->all_verts[i0 * 3 + 2];
                sum_len += sqrtf(dx * dx + dy * dy + dz * dz);
            }
        }
        m->avg_edge = (float)(sum_len / (double)(m->nt * 3));
        total_nodes += m->n_nodes;
        total_prims += m->nt;
        vo += m->nv;
        to += m->nt;
    }
    s->total_nodes = total_nodes;
    s->total_prims = total_prims;
    s->nl = xcalloc((size_t)(total_nodes ? total_nodes : 1) * 4, sizeof(float));
    s->nu = xcalloc((size_t)(total_nodes ? total_nodes : 1) * 4, sizeof(float));
    s->prim = xcalloc((size_t)(total_prims ? total_prims : 1), sizeof(uint32_t));
    s->roots = xcalloc((size_t)(nm ? nm : 1), sizeof(uint32_t));
    s->prim_off = xcalloc((size_t)(nm ? nm : 1), sizeof(uint32_t));
    s->prim_cnt = xcalloc((size_t)(nm ? nm : 1), sizeof(uint32_t));
    for (int64_t c = 0, nb = 0, pb = 0, to = 0; c < nm; c++) { /* packing, scene.cpp:287-321 */
        or_mesh* m = &s->meshes[c];
        s->roots[c] = (uint32_t)(nb + m->root);
        for (int64_t i = 0; i < m->n_nodes; i++) {
            int64_t g = nb + i;
            for (int a = 0; a < 3; a++) {
                s->nl[g * 4 + a] = m->lowers[i * 4 + a];
                s->nu[g * 4 + a] = m->uppers[i * 4 + a];
            }
            uint32_t lpk = f2u(m->lowers[i * 4 + 3]), upk = f2u(m->uppers[i * 4 + 3]);
            if ((lpk >> 30) & 3u) {
                s->nl[g * 4 + 3] = u2f(((lpk & 0x3FFFFFFFu) + (uint32_t)pb) | (1u << 30));
                s->nu[g * 4 + 3] = u2f((upk & 0x3FFFFFFFu) + (uint32_t)pb);
            } else {
                s->nl[g * 4 + 3] = u2f((lpk & 0x3FFFFFFFu) + (uint32_t)nb);
                s->nu[g * 4 + 3] = u2f((upk & 0x3FFFFFFFu) + (uint32_t)nb);
            }
        }
        for (int64_t i = 0; i < m->nt; i++) s->prim[pb + i] = m->prims[i] + (uint32_t)to;
        s->prim_off[c] = (uint32_t)pb;
        s->prim_cnt[c] = (uint32_t)m->nt;
        pb += m->nt;
        nb += m->n_nodes;
        to += m->nt;
    }
    s->finalized = 1;
    return 0;
}

int or_update_mesh(or_solver* s, int64_t mi, const float* verts, int64_t nv, const float* vels) {
    /* scene.cpp:617-696: patch vertices and velocities, refit this mesh's BVH, repack */
    if (!s->finalized || mi < 0 || mi >= s->nmesh) return -1;
    or_mesh* m = &s->meshes[mi];
    if (nv != m->nv) return -2;
    int64_t vstart = 0, nbase = 0, pbase = 0, tbase = 0;
    for (int64_t c = 0; c < mi; c++) {
        vstart += s->meshes[c].nv;
        nbase += s->meshes[c].n_nodes;
        pbase += s->meshes[c].nt;
        tbase += s->meshes[c].nt;
    }
    memcpy(s->all_verts + vstart * 3, verts, sizeof(float) * 3 * (size_t)nv);
    if (vels) memcpy(s->all_vels + vstart * 3, vels, sizeof(float) * 3 * (size_t)nv);
    else memset(s->all_vels + vstart * 3, 0, sizeof(float) * 3 * (size_t)nv);
    memcpy(m->verts, verts, sizeof(float) * 3 * (size_t)nv);
    or_bvh_refit(s->all_verts, s->all_tris + tbase * 3, m->lowers, m->uppers, m->prims, m->root);
    for (int64_t i = 0; i < m->n_nodes; i++) {
        for (int a = 0; a < 3; a++) {
            s->nl[(nbase + i) * 4 + a] = m->lowers[i * 4 + a];
            s->nu[(nbase + i) * 4 + a] = m->uppers[i * 4 + a];
        }
    }
    (void)pbase;
    return 0;
}

int or_set_particles(or_solver* s, const float* q, const float* qd, const float* w, const float* r,
                     const int32_t* flags, int64_t n) { /* scene.cpp:592-615 */
    if (n != s->n) return -1;
    for (int64_t i = 0; i < n * 3; i++) {
        s->x[i] = (real)q[i];
        s->v[i] = qd ? (real)qd[i] : RF(0.0);
    }
    if (w) for (int64_t i = 0; i < n; i++) s->w[i] = (real)w[i];
    if (r) for (int64_t i = 0; i < n; i++) s->r[i] = (real)r[i];
    if (flags) memcpy(s->flags, flags, sizeof(int32_t) * (size_t)n);
    return 0;
}

int or_set_bodies(or_solver* s, const float* q, const float* qd, const float* com, const float* I,
                  const float* invI, const float* invm, const int32_t* flags, int64_t nb) {
    if (!s->finalized || nb != s->nbody) return -1;
    for (int64_t b = 0; b < nb; b++) {
        if (q) for (int k = 0; k < 8; k++) s->body_q[b * 8 + k] = (real)q[b * 8 + k];
        if (qd) for (int k = 0; k < 8; k++) s->body_qd[b * 8 + k] = (real)qd[b * 8 + k];
        if (com) for (int k = 0; k < 3; k++) s->body_com[b * 3 + k] = (real)com[b * 3 + k];
        if (I) for (int k = 0; k < 9; k++) s->body_I[b * 9 + k] = (real)I[b * 9 + k];
        if (invI) for (int k = 0; k < 9; k++) s->body_invI[b * 9 + k] = (real)invI[b * 9 + k];
        if (invm) s->body_invm[b] = (real)invm[b];
        if (flags) s->body_flags[b] = flags[b];
    }
    s->dyn_any = 0;
    for (int64_t b = 0; b < nb; b++)
        if (s->body_invm[b] > RF(0.0)) s->dyn_any = 1;
    return 0;
}

void or_get_bodies(const or_solver* s, float* q, float* qd) {
    for (int64_t i = 0; i < s->nbody * 8; i++) {
        if (q) q[i] = (float)s->body_q[i];
        if (qd) qd[i] = (float)s->body_qd[i];
    }
}

void or_set_body_params(or_solver* s, const or_body_params* p) { s->bp = *p; }
int64_t or_rigid_contact_overflows(const or_solver* s) { return s->rc_overflow; }

static inline v3 ld3(const real* a, int64_t i) { return mk(a[i * 3], a[i * 3 + 1], a[i * 3 + 2]); }
static inline void st3(real* a, int64_t i, v3 v) { a[i * 3] = v.x; a[i * 3 + 1] = v.y; a[i * 3 + 2] = v.z; }
static inline v3 ld3f(const float* a, int64_t i) {
    return mk((real)a[i * 3], (real)a[i * 3 + 1], (real)a[i * 3 + 2]);
}

/* ------------------------------------------------------------------------- */
/* Contact generation                                                          */
/* ------------------------------------------------------------------------- */
typedef struct { int32_t part, shape; v3 bpos, bvel, nrm; } contact_t;

static void emit_contact(or_solver* s, const contact_t* c) {
    int64_t slot = s->ccount_raw++;
    if (slot >= s->cmax) return;
    s->cpart[slot] = c->part;
    s->cshape[slot] = c->shape;
    st3(s->cbpos, slot, c->bpos);
    st3(s->cbvel, slot, c->bvel);
    st3(s->cnorm, slot, c->nrm);
}

/* generate_plane_contacts.comp:27-54 */
static int plane_contact(const or_solver* s, int64_t tid, contact_t* out) {
    if ((s->flags[tid] & 1) == 0) return 0;
    v3 p = ld3(s->x, tid);
    real radius = s->r[tid];
    real alt = (real)s->cfg.ground_plane_altitude;
    real dist = p.z - alt;
    if (!(dist < (real)s->cfg.soft_contact_margin + radius)) return 0;
    out->part = (int32_t)tid;
    out->shape = 0;
    out->bpos = mk(p.x, p.y, alt);
    out->bvel = mk(RF(0.0), RF(0.0), RF(0.0));
    out->nrm = mk(RF(0.0), RF(0.0), RF(1.0));
    return 1;
}

static inline real dist_sq_aabb(v3 p, v3 lo, v3 hi) { /* generate_mesh_contacts.comp:32-35 */
    v3 d = mk(gmax(gmax(lo.x - p.x, RF(0.0)), p.x - hi.x), gmax(gmax(lo.y - p.y, RF(0.0)), p.y - hi.y),
              gmax(gmax(lo.z - p.z, RF(0.0)), p.z - hi.z));
    return vdot(d, d);
}

/* intersect_ray_tri_woop: generate_mesh_contacts.comp:77-113 */
static int intersect_ray_tri_woop(v3 p, v3 dir, v3 a, v3 b, v3 c) {
    real adir[3] = {R_FABS(dir.x), R_FABS(dir.y), R_FABS(dir.z)};
    real dv[3] = {dir.x, dir.y, dir.z};
    int kz = 0;
    if (adir[1] > adir[0]) kz = 1;
    if (adir[2] > (kz == 1 ? adir[1] : adir[0])) kz = 2;
    int kx = kz + 1;
    if (kx == 3) kx = 0;
    int ky = kx + 1;
    if (ky == 3) ky = 0;
    if (dv[kz] < RF(0.0)) { int t = kx; kx = ky; ky = t; }
    real Sx = dv[kx] / dv[kz], Sy = dv[ky] / dv[kz], Sz = RF(1.0) / dv[kz];
    v3 A3 = vsub(a, p), B3 = vsub(b, p), C3 = vsub(c, p);
    real A[3] = {A3.x, A3.y, A3.z}, B[3] = {B3.x, B3.y, B3.z}, C[3] = {C3.x, C3.y, C3.z};
    real Ax = A[kx] - Sx * A[kz], Ay = A[ky] - Sy * A[kz];
    real Bx = B[kx] - Sx * B[kz], By = B[ky] - Sy * B[kz];
    real Cx = C[kx] - Sx * C[kz], Cy = C[ky] - Sy * C[kz];
    real U = diff_product(Cx, By, Cy, Bx);
    real V = diff_product(Ax, Cy, Ay, Cx);
    real W = diff_product(Bx, Ay, By, Ax);
    if ((U < RF(0.0) || V < RF(0.0) || W < RF(0.0)) && (U > RF(0.0) || V > RF(0.0) || W > RF(0.0))) return 0;
    real det = U + V + W;
    if (det == RF(0.0)) return 0;
    real Az = Sz * A[kz], Bz = Sz * B[kz], Cz = Sz * C[kz];
    real T = U * Az + V * Bz + W * Cz;
    if ((T < RF(0.0) && det > RF(0.0)) || (T > RF(0.0) && det < RF(0.0))) return 0;
    return 1;
}

/* closest_point_triangle: generate_mesh_contacts.comp:115-179 */
static void closest_point_triangle(v3 p, v3 a, v3 b, v3 c, v3* cp, v3* tri_normal, v3* bary) {
    v3 ab = vsub(b, a), ac = vsub(c, a), ap = vsub(p, a);
    *tri_normal = vnormalize(vcross(ab, ac));
    real u, v;
    real d1 = exact_dot(ab, ap), d2 = exact_dot(ac, ap);
    if (d1 <= RF(0.0) && d2 <= RF(0.0)) {
        v = RF(0.0);
        u = RF(1.0);
    } else {
        v3 bp = vsub(p, b);
        real d3 = exact_dot(ab, bp), d4 = exact_dot(ac, bp);
        if (d3 >= RF(0.0) && d4 <= d3) {
            v = RF(1.0);
            u = RF(0.0);
        } else {
            real vc = R_FMA(d1, d4, -(d2 * d3));
            if (vc <= RF(0.0) && d1 >= RF(0.0) && d3 <= RF(0.0)) {
                v = exact_div1(d1, d1 - d3);
                u = RF(1.0) - v;
            } else {
                v3 cp_p = vsub(p, c);
                real d5 = exact_dot(ab, cp_p), d6 = exact_dot(ac, cp_p);
                if (d6 >= RF(0.0) && d5 <= d6) {
                    v = RF(0.0);
                    u = RF(0.0);
                } else {
                    real vb = R_FMA(d5, d2, -(d1 * d6));
                    if (vb <= RF(0.0) && d2 >= RF(0.0) && d6 <= RF(0.0)) {
                        real w_val = exact_div1(d2, d2 - d6);
                        v = RF(0.0);
                        u = RF(1.0) - w_val;
                    } else {
                        real va = R_FMA(d3, d6, -(d5 * d4));
                        if (va <= RF(0.0) && (d4 - d3) >= RF(0.0) && (d5 - d6) >= RF(0.0)) {
                            real w_val = exact_div1(d4 - d3, (d4 - d3) + (d5 - d6));
                            v = RF(1.0) - w_val;
                            u = (RF(1.0) - v) - w_val;
                        } else {
                            real sum_vavb = va + vb;
                            real sum_all = vc + sum_vavb;
                            real r0 = RF(1.0) / sum_all;
                            real rem = R_FMA(-sum_all, r0, RF(1.0));
                            real denom = R_FMA(rem, r0, r0);
                            v = vb * denom;
                            u = R_FMA(-vc, denom, RF(1.0) - v);
                        }
                    }
                }
            }
        }
    }
    real w_out = (RF(1.0) - u) - v;
    *bary = mk(u, v, w_out);
    *cp = vadd(vadd(vmuls(a, u), vmuls(b, v)), vmuls(c, w_out));
}

void or_closest_point_triangle(const float* p, const float* a, const float* b, const float* c,
                               float* cp, float* tn, float* bary) {
    v3 o, n, br;
    closest_point_triangle(mk(p[0], p[1], p[2]), mk(a[0], a[1], a[2]), mk(b[0], b[1], b[2]),
                           mk(c[0], c[1], c[2]), &o, &n, &br);
    cp[0] = (float)o.x; cp[1] = (float)o.y; cp[2] = (float)o.z;
    tn[0] = (float)n.x; tn[1] = (float)n.y; tn[2] = (float)n.z;
    bary[0] = (float)br.x; bary[1] = (float)br.y; bary[2] = (float)br.z;
}

static inline v3 vert(const or_solver* s, uint32_t t, int k) {
    return ld3f(s->all_verts, s->all_tris[t * 3 + k]);
}

/* generate_mesh_contacts.comp:181-414, one particle, appends up to nmesh contacts */
/* Closest-point query of point p (in the mesh's own frame) against mesh ci, the
 * per-mesh body of generate_mesh_contacts.comp:197-411: returns 1 and the contact's
 * surface point, surface velocity and normal when the mesh is within
 * margin + shape margin + radius. */
static int mesh_query(const or_solver* s, int64_t ci, v3 p, real radius, real margin, v3* o_bpos, v3* o_bvel,
                      v3* o_nrm, int* stack_overflow) {
    real avg_edge = (real)s->meshes[0].avg_edge;
    real eps_md = avg_edge * RF(1e-3);
    real eps2 = eps_md * eps_md;
    const real PI_ = RF(3.14159265359);
    {
        real max_dist = margin + (real)s->meshes[ci].margin + radius;
        uint32_t stack[32];
        uint32_t sp = 0;
        stack[sp++] = s->roots[ci];
        real min_dist = max_dist;
        v3 acc_normal = mk(RF(0.0), RF(0.0), RF(0.0));
        uint32_t min_face = 0;
        real sv_v = RF(0.0), sv_w = RF(0.0);
        int found = 0;
        int wt = s->meshes[ci].watertight;
        real min_dist_sq = max_dist * max_dist;
        while (sp > 0) {
            uint32_t ni = stack[--sp];
            v3 lo = mk(s->nl[ni * 4], s->nl[ni * 4 + 1], s->nl[ni * 4 + 2]);
            v3 hi = mk(s->nu[ni * 4], s->nu[ni * 4 + 1], s->nu[ni * 4 + 2]);
            real nds = dist_sq_aabb(p, lo, hi);
            if (wt) {
                if (nds > min_dist_sq) continue;
            } else {
                if (nds > (min_dist + eps_md) * (min_dist + eps_md)) continue;
            }
            uint32_t lpk = f2u(s->nl[ni * 4 + 3]);
            uint32_t left_i = lpk & 0x3FFFFFFFu, is_leaf = (lpk >> 30) & 3u;
            uint32_t right_i = f2u(s->nu[ni * 4 + 3]) & 0x3FFFFFFFu;
            if (is_leaf) {
                for (uint32_t pc = left_i; pc < right_i; pc++) {
                    uint32_t t = s->prim[pc];
                    v3 a = vert(s, t, 0), b = vert(s, t, 1), c = vert(s, t, 2);
                    v3 e0 = vsub(b, a), e1 = vsub(c, a), e2 = vsub(c, b);
                    v3 normal = vcross(e0, e1);
                    real e0n = vdot(e0, e0), e1n = vdot(e1, e1), e2n = vdot(e2, e2);
                    if (vlength(normal) / (e0n + e1n + e2n) < RF(1.0e-6)) continue;
                    v3 cp, tn, tb;
                    closest_point_triangle(p, a, b, c, &cp, &tn, &tb);
                    if (wt) {
                        v3 diff = vsub(cp, p);
                        real dist_sq = vdot(diff, diff);
                        if (dist_sq < min_dist_sq) {
                            min_dist_sq = dist_sq;
                            min_face = t;
                            sv_v = tb.y;
                            sv_w = tb.z;
                            found = 1;
                        }
                    } else {
                        real dist = exact_length(vsub(cp, p));
                        if (dist < min_dist + eps_md) {
                            real weight;
                            v3 cp_p = vsub(cp, a), cq_p = vsub(cp, b), cr_p = vsub(cp, c);
                            real lcp = vdot(cp_p, cp_p), lcq = vdot(cq_p, cq_p), lcr = vdot(cr_p, cr_p);
                            if (lcp < eps2) {
                                weight = r_acos(gclamp(vdot(vnormalize(e0), vnormalize(e1)), RF(-1.0), RF(1.0)));
                            } else if (lcq < eps2) {
                                weight = r_acos(gclamp(vdot(vnormalize(e2), vnormalize(vneg(e0))), RF(-1.0), RF(1.0)));
                            } else if (lcr < eps2) {
                                weight = r_acos(gclamp(vdot(vnormalize(vneg(e1)), vnormalize(vneg(e2))), RF(-1.0), RF(1.0)));
                            } else {
                                real e0cp = vdot(e0, cp_p), e2cq = vdot(e2, cq_p), e1cp = vdot(e1, cp_p);
                                if ((lcp * e0n - e0cp * e0cp < eps2 * e0n) || (lcq * e2n - e2cq * e2cq < eps2 * e2n) ||
                                    (lcp * e1n - e1cp * e1cp < eps2 * e1n))
                                    weight = PI_;
                                else
                                    weight = RF(2.0) * PI_;
                            }
                            if (dist > min_dist - eps_md) {
                                acc_normal = vadd(acc_normal, vmuls(tn, weight));
                                if (dist < min_dist) {
                                    min_dist = dist;
                                    min_face = t;
                                    sv_v = tb.y;
                                    sv_w = tb.z;
                                }
                            } else {
                                min_dist = dist;
                                min_face = t;
                                sv_v = tb.y;
                                sv_w = tb.z;
                                acc_normal = vmuls(tn, weight);
                            }
                            found = 1;
                        }
                    }
                }
            } else {
                v3 llo = mk(s->nl[left_i * 4], s->nl[left_i * 4 + 1], s->nl[left_i * 4 + 2]);
                v3 lhi = mk(s->nu[left_i * 4], s->nu[left_i * 4 + 1], s->nu[left_i * 4 + 2]);
                v3 rlo = mk(s->nl[right_i * 4], s->nl[right_i * 4 + 1], s->nl[right_i * 4 + 2]);
                v3 rhi = mk(s->nu[right_i * 4], s->nu[right_i * 4 + 1], s->nu[right_i * 4 + 2]);
                real lds = dist_sq_aabb(p, llo, lhi), rds = dist_sq_aabb(p, rlo, rhi);
                real thresh = wt ? min_dist_sq : ((min_dist + eps_md) * (min_dist + eps_md));
                /* the shader's stack is 32 deep with no check; a push past it is
                 * undefined there and is counted (and dropped) here */
                if (lds < rds) {
                    if (rds < thresh) { if (sp < 32) stack[sp++] = right_i; else *stack_overflow = 1; }
                    if (lds < thresh) { if (sp < 32) stack[sp++] = left_i; else *stack_overflow = 1; }
                } else {
                    if (lds < thresh) { if (sp < 32) stack[sp++] = left_i; else *stack_overflow = 1; }
                    if (rds < thresh) { if (sp < 32) stack[sp++] = right_i; else *stack_overflow = 1; }
                }
            }
        }
        if (wt) min_dist = exact_sqrt(min_dist_sq);
        if (found && min_dist < max_dist) {
            real u_mesh = (RF(1.0) - sv_v) - sv_w;
            real v_mesh = sv_v;
            v3 v0 = vert(s, min_face, 0), v1 = vert(s, min_face, 1), v2 = vert(s, min_face, 2);
            real w_eval = (RF(1.0) - u_mesh) - v_mesh;
            v3 term_b = vmuls(v1, v_mesh);
            v3 term_ab = vfma_vs(v0, u_mesh, term_b);
            v3 shape_p = vfma_vs(v2, w_eval, term_ab);
            uint32_t i0 = s->all_tris[min_face * 3], i1 = s->all_tris[min_face * 3 + 1],
                     i2 = s->all_tris[min_face * 3 + 2];
            v3 vel0 = ld3f(s->all_vels, i0), vel1 = ld3f(s->all_vels, i1), vel2 = ld3f(s->all_vels, i2);
            v3 vt_b = vmuls(vel1, v_mesh);
            v3 vt_ab = vfma_vs(vel0, u_mesh, vt_b);
            v3 shape_v = vfma_vs(vel2, w_eval, vt_ab);
            real sign;
            if (wt) {
                v3 ray_dir = mk(RF(1.029700994), RF(1.086472273), RF(1.034694910));
                uint32_t hits = 0;
                uint32_t po = s->prim_off[ci], pn = s->prim_cnt[ci];
                for (uint32_t ti = 0; ti < pn; ti++) {
                    uint32_t t = s->prim[po + ti];
                    if (intersect_ray_tri_woop(p, ray_dir, vert(s, t, 0), vert(s, t, 1), vert(s, t, 2))) hits++;
                }
                sign = (hits & 1u) ? RF(-1.0) : RF(1.0);
            } else {
                sign = vdot(acc_normal, vsub(p, shape_p)) > RF(0.0) ? RF(1.0) : RF(-1.0);
            }
            v3 delta = vsub(p, shape_p);
            real delta_len = exact_length(delta);
            v3 nrm = delta_len > RF(0.0) ? vmuls(exact_div(delta, delta_len), sign) : mk(RF(0.0), RF(0.0), RF(1.0));
            real d = delta_len * sign;
            *o_bpos = vfma_vs(vneg(nrm), d, p);
            *o_bvel = shape_v;
            *o_nrm = nrm;
            return 1;
        }
    }
    return 0;
}

static inline int posed(const or_solver* s, int64_t b) { return s->dyn_any && s->body_invm[b] > RF(0.0); }

static void body_state(const real* q, int64_t b, v3* pos, q4* rot) {
    *pos = mk(q[b * 8], q[b * 8 + 1], q[b * 8 + 2]);
    rot->x = q[b * 8 + 4];
    rot->y = q[b * 8 + 5];
    rot->z = q[b * 8 + 6];
    rot->w = q[b * 8 + 7];
}

/* generate_mesh_contacts.comp:197-411 for every mesh, in index order. A mesh whose
 * body is dynamic holds its vertices in the body frame: the particle is taken into
 * that frame with the inverse of the pose the solve applies
 * (solve_particle_shape_contacts.comp:134), the contact point and surface velocity
 * stay in the body frame (the solve transforms them, :134 and :155) and the normal
 * is rotated to world space (the solve reads it as is, :138). */
static int mesh_contacts(const or_solver* s, int64_t tid, contact_t* out, int* stack_overflow) {
    int nout = 0;
    if ((s->flags[tid] & 1) == 0) return 0;
    v3 p = ld3(s->x, tid);
    real radius = s->r[tid];
    for (int64_t ci = 0; ci < s->nmesh; ci++) {
        v3 q = p, bpos, bvel, nrm;
        v3 pos;
        q4 rot;
        int pz = posed(s, ci);
        if (pz) {
            body_state(s->body_q, ci, &pos, &rot);
            q = quat_rotate_inv(rot, vsub(p, pos));
        }
        if (!mesh_query(s, ci, q, radius, (real)s->cfg.soft_contact_margin, &bpos, &bvel, &nrm, stack_overflow))
            continue;
        contact_t* c = &out[nout++];
        c->part = (int32_t)tid;
        c->shape = (int32_t)ci + 1;
        c->bpos = bpos;
        c->bvel = bvel;
        c->nrm = pz ? quat_rotate(rot, nrm) : nrm;
    }
    return nout;
}

static void collide(or_solver* s) { /* scene.cpp:848-861 */
    s->ccount_raw = 0;
    int64_t n = s->n;
    if (s->cfg.has_ground_plane) {
        for (int64_t i = 0; i < n; i++) {
            contact_t c;
            if (plane_contact(s, i, &c)) emit_contact(s, &c);
        }
    }
    if (s->nmesh > 0) {
        /* per-particle work in parallel; each thread takes a contiguous particle
         * block so that concatenating thread buffers in thread order gives the
         * canonical (particle, mesh) order */
        int nt = or_get_threads();
        contact_t** bufs = xcalloc((size_t)nt, sizeof(contact_t*));
        int64_t* lens = xcalloc((size_t)nt, sizeof(int64_t));
        int ovf = 0;
#ifdef _OPENMP
#pragma omp parallel OMP_THREADS reduction(| : ovf)
#endif
        {
#ifdef _OPENMP
            int t = omp_get_thread_num(), T = omp_get_num_threads();
#else
            int t = 0, T = 1;
#endif
            int64_t b0 = n * t / T, b1 = n * (t + 1) / T;
            int64_t cap = 64, len = 0;
            contact_t* buf = xcalloc((size_t)cap, sizeof(contact_t));
            contact_t* tmp = xcalloc((size_t)s->nmesh, sizeof(contact_t));
            for (int64_t i = b0; i < b1; i++) {
                int k = mesh_contacts(s, i, tmp, &ovf);
                if (len + k > cap) {
                    while (len + k > cap) cap *= 2;
                    buf = realloc(buf, sizeof(contact_t) * (size_t)cap);
                }
                memcpy(buf + len, tmp, sizeof(contact_t) * (size_t)k);
                len += k;
            }
            free(tmp);
            if (t < nt) { bufs[t] = buf; lens[t] = len; } else free(buf);
        }
        for (int t = 0; t < nt; t++) {
            for (int64_t k = 0; k < lens[t]; k++) emit_contact(s, &bufs[t][k]);
            free(bufs[t]);
        }
        free(bufs);
        free(lens);
        if (ovf) fprintf(stderr, "oracle: BVH traversal stack overflow (push dropped)\n");
    }
}

/* ------------------------------------------------------------------------- */
/* Integrate, hash grid, sort, offsets                                         */
/* ------------------------------------------------------------------------- */
static void integrate(or_solver* s, real dt) { /* integrate_particles.comp:26-60 */
    real vmax = (real)s->cfg.particle_v_max;
    v3 g = mk((real)s->cfg.gravity[0], (real)s->cfg.gravity[1], (real)s->cfg.gravity[2]);
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int64_t i = 0; i < s->n; i++) {
        v3 x0 = ld3(s->x, i), v0 = ld3(s->v, i);
        st3(s->x0, i, x0);
        st3(s->v0, i, v0);
        if ((s->flags[i] & 1) == 0) continue;
        v3 f0 = mk(RF(0.0), RF(0.0), RF(0.0)); /* external force buffer is all zero (scene.cpp:82-83) */
        real inv_mass = s->w[i];
        real g_scale = inv_mass > RF(0.0) ? RF(1.0) : RF(0.0);
        v3 v1 = vadd(v0, vmuls(vadd(vmuls(f0, inv_mass), vmuls(g, g_scale)), dt));
        real v1_mag = vlength(v1);
        if (v1_mag > vmax) v1 = vmuls(v1, vmax / v1_mag);
        v3 x1 = vadd(x0, vmuls(v1, dt));
        st3(s->x, i, x1);
        st3(s->v, i, v1);
    }
}

static inline int32_t imax0(int32_t a) { return a < 0 ? 0 : a; }
static uint32_t hash_grid_index(v3 p, real inv) { /* grid_cell_indices.comp:17-25 */
    int32_t gx = f2i(R_FLOOR(p.x * inv)), gy = f2i(R_FLOOR(p.y * inv)), gz = f2i(R_FLOOR(p.z * inv));
    gx = imax0(gx + (1 << 20));
    gy = imax0(gy + (1 << 20));
    gz = imax0(gz + (1 << 20));
    return (uint32_t)((gz % 128) * (128 * 128) + (gy % 128) * 128 + (gx % 128));
}

static void build_grid(or_solver* s, real inv) {
    int64_t n = s->n;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int64_t i = 0; i < n; i++) {
        s->cells[i] = hash_grid_index(ld3(s->x, i), inv);
        s->ids[i] = (uint32_t)i;
    }
    /* stable sort by cell, ties by id (gpu_sort.h:110-129 + sort_scatter.comp:58-63):
     * a counting sort over the 2^21 cells; cend doubles as the bucket counter */
    memset(s->cstart, 0, sizeof(int32_t) * NUM_CELLS);
    memset(s->cend, 0, sizeof(int32_t) * NUM_CELLS);
    for (int64_t i = 0; i < n; i++) s->cend[s->cells[i]]++;
    int32_t run = 0;
    for (int c = 0; c < NUM_CELLS; c++) {
        int32_t k = s->cend[c];
        s->cend[c] = run;
        run += k;
    }
    for (int64_t i = 0; i < n; i++) {
        uint32_t c = s->cells[i];
        int32_t pos = s->cend[c]++;
        s->scells[pos] = c;
        s->sids[pos] = (uint32_t)i;
    }
    /* grid_offsets.comp:16-34 after the zero fills of scene.cpp:918-922 */
    memset(s->cstart, 0, sizeof(int32_t) * NUM_CELLS);
    memset(s->cend, 0, sizeof(int32_t) * NUM_CELLS);
    for (int64_t t = 0; t < n; t++) {
        int32_t c = (int32_t)s->scells[t];
        if (t == 0) {
            s->cstart[c] = 0;
        } else {
            int32_t p = (int32_t)s->scells[t - 1];
            if (c != p) {
                s->cstart[c] = (int32_t)t;
                s->cend[p] = (int32_t)t;
            }
        }
        if (t == n - 1) s->cend[c] = (int32_t)t + 1;
    }
}

/* ------------------------------------------------------------------------- */
/* Solve                                                                       */
/* ------------------------------------------------------------------------- */
static void body_pose(const or_solver* s, int32_t b, v3* pos, q4* rot, v3* com) {
    if (b >= 0) {
        *pos = mk(s->body_q[b * 8], s->body_q[b * 8 + 1], s->body_q[b * 8 + 2]);
        rot->x = s->body_q[b * 8 + 4];
        rot->y = s->body_q[b * 8 + 5];
        rot->z = s->body_q[b * 8 + 6];
        rot->w = s->body_q[b * 8 + 7];
        *com = ld3(s->body_com, b);
    } else {
        *pos = mk(RF(0.0), RF(0.0), RF(0.0));
        rot->x = rot->y = rot->z = RF(0.0);
        rot->w = RF(1.0);
        *com = mk(RF(0.0), RF(0.0), RF(0.0));
    }
}

/* solve_particle_shape_contacts.comp:104-200 for one contact slot; adds into delta */
static void shape_contact(or_solver* s, int64_t tid, const real* X, const real* V, real dt) {
    int32_t shape = s->cshape[tid];
    int32_t body = s->shape_body[shape];
    int32_t pi = s->cpart[tid];
    int32_t pflag = s->flags[pi];
    if ((pflag & 1) == 0) return;
    if (pflag & 2) {
        if (body < 0) return;
        if (s->body_flags[body] & 4) return;
        if (s->body_invm[body] == RF(0.0)) return;
    }
    v3 px = ld3(X, pi), pv = ld3(V, pi);
    v3 X_pos, X_com;
    q4 X_rot;
    body_pose(s, body, &X_pos, &X_rot, &X_com);
    v3 bx = vadd(X_pos, quat_rotate(X_rot, ld3(s->cbpos, tid)));
    v3 r = vsub(bx, vadd(X_pos, quat_rotate(X_rot, X_com)));
    v3 n = ld3(s->cnorm, tid);
    v3 d_px = vsub(px, bx);
    real c = R_FMA(n.z, d_px.z, R_FMA(n.x, d_px.x, n.y * d_px.y)) - s->r[pi];
    if (c > (real)s->cfg.particle_adhesion) return;
    real mu = RF(0.5) * ((real)s->cfg.soft_contact_mu + s->shape_mu[shape]);
    v3 body_v = mk(RF(0.0), RF(0.0), RF(0.0)), body_w = body_v;
    if (body >= 0) {
        body_v = mk(s->body_qd[body * 8], s->body_qd[body * 8 + 1], s->body_qd[body * 8 + 2]);
        body_w = mk(s->body_qd[body * 8 + 4], s->body_qd[body * 8 + 5], s->body_qd[body * 8 + 6]);
    }
    v3 bv = vadd(vadd(body_v, vcross(body_w, r)), quat_rotate(X_rot, ld3(s->cbvel, tid)));
    v3 v = vsub(pv, bv);
    real lambda_n = c;
    v3 delta_n = vmuls(n, lambda_n);
    real vn = n.y * v.y;
    vn = R_FMA(n.x, v.x, vn);
    vn = R_FMA(n.z, v.z, vn);
    v3 vt = mk(R_FMA(-n.x, vn, v.x), R_FMA(-n.y, vn, v.y), R_FMA(-n.z, vn, v.z));
    real w1 = s->w[pi], w2 = RF(0.0);
    if (body >= 0) {
        v3 ang = vcross(r, n);
        v3 ra = quat_rotate_inv(X_rot, ang);
        const real* M = &s->body_invI[body * 9];
        v3 Mra = mk((M[0] * ra.x + M[1] * ra.y) + M[2] * ra.z, (M[3] * ra.x + M[4] * ra.y) + M[5] * ra.z,
                    (M[6] * ra.x + M[7] * ra.y) + M[8] * ra.z);
        w2 = s->body_invm[body] + vdot(ra, Mra);
    }
    real denom = w1 + w2;
    if (denom == RF(0.0)) return;
    real vt_len = exact_length(vt);
    real lambda_f = gmax(mu * lambda_n, -vt_len * dt);
    v3 vt_dir = vt_len > RF(0.0) ? exact_div(vt, vt_len) : mk(RF(0.0), RF(0.0), RF(0.0));
    v3 diff = mk(R_FMA(vt_dir.x, lambda_f, -delta_n.x), R_FMA(vt_dir.y, lambda_f, -delta_n.y),
                 R_FMA(vt_dir.z, lambda_f, -delta_n.z));
    v3 delta_total = vmuls(exact_div(diff, denom), (real)s->cfg.soft_contact_relaxation);
    v3 fd = mk(w1 * delta_total.x, w1 * delta_total.y, w1 * delta_total.z);
    s->delta[pi * 3 + 0] += fd.x;
    s->delta[pi * 3 + 1] += fd.y;
    s->delta[pi * 3 + 2] += fd.z;
    if (body >= 0 && s->body_invm[body] > RF(0.0)) { /* :193-199, kept per slot and summed per body later */
        v3 delta_v = mk(delta_total.x / dt, delta_total.y / dt, delta_total.z / dt);
        v3 delta_w = vcross(r, delta_v);
        real* o = &s->bdel[tid * 6];
        o[0] = -delta_v.x; o[1] = -delta_v.y; o[2] = -delta_v.z;
        o[3] = -delta_w.x; o[4] = -delta_w.y; o[5] = -delta_w.z;
        s->bvalid[tid] = 1;
    }
}

static inline int32_t cell_index(int32_t x, int32_t y, int32_t z) { /* pp shader :67-79 */
    x += 1 << 20;
    y += 1 << 20;
    z += 1 << 20;
    x = imax0(x);
    y = imax0(y);
    z = imax0(z);
    return (z % 128) * (128 * 128) + (y % 128) * 128 + (x % 128);
}

/* solve_particle_particle_contacts.comp:107-218 for sorted slot tid; returns the
 * total added to delta[i] (or nothing for inactive particles) */
static void pp_contact(or_solver* s, int64_t tid, const real* X, const real* V, real dt, real inv) {
    int32_t i = (int32_t)s->sids[tid];
    int32_t pflag = s->flags[i];
    if ((pflag & 1) == 0) return;
    int32_t is_proxy = pflag & 2;
    v3 x = ld3(X, i), v = ld3(V, i);
    real radius = s->r[i], w1 = s->w[i];
    real k_mu = (real)s->cfg.particle_mu, k_coh = (real)s->cfg.particle_cohesion;
    real R = radius + (real)s->cfg.particle_max_radius + k_coh;
    int32_t xs = f2i(R_FLOOR((x.x - R) * inv)), ys = f2i(R_FLOOR((x.y - R) * inv)), zs = f2i(R_FLOOR((x.z - R) * inv));
    int32_t xe = f2i(R_FLOOR((x.x + R) * inv)), ye = f2i(R_FLOOR((x.y + R) * inv)), ze = f2i(R_FLOOR((x.z + R) * inv));
    if (xe > xs + GRID_DIM - 1) xe = xs + GRID_DIM - 1;
    if (ye > ys + GRID_DIM - 1) ye = ys + GRID_DIM - 1;
    if (ze > zs + GRID_DIM - 1) ze = zs + GRID_DIM - 1;
    v3 delta = mk(RF(0.0), RF(0.0), RF(0.0));
    for (int32_t cz = zs; cz <= ze; cz++)
        for (int32_t cy = ys; cy <= ye; cy++)
            for (int32_t cx = xs; cx <= xe; cx++) {
                int32_t cell = cell_index(cx, cy, cz);
                int32_t st = s->cstart[cell], en = s->cend[cell];
                for (int32_t k = st; k < en; k++) {
                    int32_t j = (int32_t)s->sids[k];
                    if (j == i) continue;
                    int32_t nflag = s->flags[j];
                    if ((nflag & 1) == 0) continue;
                    if (is_proxy != 0 && (((nflag & 2) != 0) || (s->w[j] <= RF(0.0)))) continue;
                    v3 raw = vsub(x, ld3(X, j));
                    if (R_FABS(raw.x) > R || R_FABS(raw.y) > R || R_FABS(raw.z) > R) continue;
                    v3 nn = raw;
                    real d = exact_length(nn);
                    real err = d - radius - s->r[j];
                    if (err > k_coh || d <= RF(0.0)) continue;
                    real w2 = s->w[j];
                    real denom = w1 + w2;
                    if (denom <= RF(0.0)) continue;
                    nn = exact_div(nn, d);
                    v3 vrel = vsub(v, ld3(V, j));
                    real lambda_n = err;
                    real vn = exact_dot(nn, vrel);
                    v3 vt = mk(R_FMA(vn, -nn.x, vrel.x), R_FMA(vn, -nn.y, vrel.y), R_FMA(vn, -nn.z, vrel.z));
                    real vt_len = exact_length(vt);
                    real lambda_f = gmax(k_mu * lambda_n, -vt_len * dt);
                    v3 vt_dir = vt_len > RF(0.0) ? exact_div(vt, vt_len) : mk(RF(0.0), RF(0.0), RF(0.0));
                    v3 p2 = vmuls(nn, err);
                    v3 diff = mk(R_FMA(vt_dir.x, lambda_f, -p2.x), R_FMA(vt_dir.y, lambda_f, -p2.y),
                                 R_FMA(vt_dir.z, lambda_f, -p2.z));
                    delta = vadd(delta, exact_div(diff, denom));
                }
            }
    real relax = (real)s->cfg.soft_contact_relaxation;
    v3 dw = mk(R_FMA(delta.x, w1, RF(0.0)), R_FMA(delta.y, w1, RF(0.0)), R_FMA(delta.z, w1, RF(0.0)));
    v3 total = mk(R_FMA(dw.x, relax, RF(0.0)), R_FMA(dw.y, relax, RF(0.0)), R_FMA(dw.z, relax, RF(0.0)));
    s->delta[i * 3 + 0] += total.x;
    s->delta[i * 3 + 1] += total.y;
    s->delta[i * 3 + 2] += total.z;
}

/* apply_particle_deltas.comp:38-58. Inactive particles keep their predicted state
 * (the shader writes nothing for them, leaving the output buffer stale). */
static void apply_deltas(or_solver* s, const real* XP, const real* VP, real dt) {
    real vmax = (real)s->cfg.particle_v_max;
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static)
#endif
    for (int64_t i = 0; i < s->n; i++) {
        if ((s->flags[i] & 1) == 0) {
            st3(s->xo, i, ld3(XP, i));
            st3(s->vo, i, ld3(VP, i));
            continue;
        }
        v3 x0 = ld3(s->x0, i), xp = ld3(XP, i), d = ld3(s->delta, i);
        v3 x_new = vadd(xp, d);
        v3 v_new = exact_div_apply(vsub(x_new, x0), dt);
        real v_mag = vlength(v_new);
        if (v_mag > vmax) {
            v_new = vmuls(v_new, vmax / v_mag);
            x_new = vadd(x0, vmuls(v_new, dt));
        }
        st3(s->xo, i, x_new);
        st3(s->vo, i, v_new);
    }
}

/* apply_particle_shape_restitution.comp:248-316 for one slot, with the
 * pre-restitution velocity snapshot vsnap */
static void restitution_contact(or_solver* s, int64_t tid) {
    int32_t shape = s->cshape[tid];
    int32_t body = s->shape_body[shape];
    int32_t pi = s->cpart[tid];
    if ((s->flags[pi] & 1) == 0) return;
    v3 v_new = ld3(s->vsnap, pi), px = ld3(s->x0, pi), v_old = ld3(s->v0, pi);
    v3 X_pos, X_com;
    q4 X_rot;
    body_pose(s, body, &X_pos, &X_rot, &X_com);
    /* body_q_prev is bound to body_q (scene.cpp:577-580) while every body is static;
     * with dynamic bodies it is the state at the start of the substep */
    v3 X_pos_prev = X_pos;
    q4 X_rot_prev = X_rot;
    if (s->dyn_any && body >= 0) body_state(s->body_qp, body, &X_pos_prev, &X_rot_prev);
    v3 c_bpos = ld3(s->cbpos, tid);
    v3 bx = vadd(X_pos, quat_rotate(X_rot, c_bpos));
    v3 n = ld3(s->cnorm, tid);
    v3 d_px = vsub(px, bx);
    real c = R_FMA(n.z, d_px.z, R_FMA(n.x, d_px.x, n.y * d_px.y)) - s->r[pi];
    if (c > (real)s->cfg.particle_adhesion) return;
    v3 bx_prev = vadd(X_pos_prev, quat_rotate(X_rot_prev, c_bpos));
    v3 r = vsub(bx_prev, vadd(X_pos_prev, quat_rotate(X_rot_prev, X_com)));
    v3 bv_contact = quat_rotate(X_rot_prev, ld3(s->cbvel, tid));
    v3 bv_old = bv_contact, bv_new = bv_contact;
    if (body >= 0) {
        const real* qdo = s->dyn_any ? s->body_qdp : s->body_qd;
        v3 bvo = mk(qdo[body * 8], qdo[body * 8 + 1], qdo[body * 8 + 2]);
        v3 bwo = mk(qdo[body * 8 + 4], qdo[body * 8 + 5], qdo[body * 8 + 6]);
        v3 bvn = mk(s->body_qd[body * 8], s->body_qd[body * 8 + 1], s->body_qd[body * 8 + 2]);
        v3 bwn = mk(s->body_qd[body * 8 + 4], s->body_qd[body * 8 + 5], s->body_qd[body * 8 + 6]);
        bv_old = vadd(vadd(bvo, vcross(bwo, r)), bv_contact);
        bv_new = vadd(vadd(bvn, vcross(bwn, r)), bv_contact);
    }
    v3 vdo = vsub(v_old, bv_old);
    real rel_old = R_FMA(n.z, vdo.z, R_FMA(n.y, vdo.y, n.x * vdo.x));
    v3 vdn = vsub(v_new, bv_new);
    real rel_new = R_FMA(n.z, vdn.z, R_FMA(n.x, vdn.x, n.y * vdn.y));
    if (rel_old < RF(0.0)) {
        real rt = gmax((-(real)s->cfg.soft_contact_restitution) * rel_old, RF(0.0));
        real scalar = (-rel_new) + rt;
        s->v[pi * 3 + 0] += n.x * scalar;
        s->v[pi * 3 + 1] += n.y * scalar;
        s->v[pi * 3 + 2] += n.z * scalar;
    }
}

/* ------------------------------------------------------------------------- */
/* Rigid bodies (extension). Body math follows integrate_bodies.comp,          */
/* apply_body_deltas.comp and solve_body_contact_positions.comp, which the     */
/* reference compiles but never dispatches; their Warp-convention quaternion    */
/* helpers are restated here as written there.                                 */
/* ------------------------------------------------------------------------- */
static inline v3 wq_rot(q4 q, v3 v) { /* v + 2*cross(q.xyz, cross(q.xyz, v) + v*q.w), integrate_bodies.comp:66-69 */
    v3 qv = mk(q.x, q.y, q.z);
    v3 t = vadd(vcross(qv, v), vmuls(v, q.w));
    return vadd(v, vmuls(vcross(qv, t), RF(2.0)));
}
static inline v3 wq_rot_inv(q4 q, v3 v) { /* integrate_bodies.comp:71-73 */
    q4 c = q;
    c.x = -q.x;
    c.y = -q.y;
    c.z = -q.z;
    return wq_rot(c, v);
}
static inline q4 wq_mul(q4 p, q4 q) { /* integrate_bodies.comp:57-63 */
    q4 r;
    v3 c = vcross(mk(p.x, p.y, p.z), mk(q.x, q.y, q.z));
    r.w = p.w * q.w - vdot(mk(p.x, p.y, p.z), mk(q.x, q.y, q.z));
    r.x = (p.w * q.x + q.w * p.x) + c.x;
    r.y = (p.w * q.y + q.w * p.y) + c.y;
    r.z = (p.w * q.z + q.w * p.z) + c.z;
    return r;
}
static inline q4 q_axpy(q4 a, q4 b, real s) { /* a + b * s */
    q4 r;
    r.x = a.x + b.x * s;
    r.y = a.y + b.y * s;
    r.z = a.z + b.z * s;
    r.w = a.w + b.w * s;
    return r;
}
static inline q4 q_normalize(q4 a) { /* normalize(vec4) = v / length(v), IEEE sqrt and division */
    real l = R_SQRT(((a.x * a.x + a.y * a.y) + a.z * a.z) + a.w * a.w);
    q4 r;
    r.x = a.x / l;
    r.y = a.y / l;
    r.z = a.z / l;
    r.w = a.w / l;
    return r;
}
/* 3x3 times vector, 9 floats column-major: col0*v.x + col1*v.y + col2*v.z (integrate_bodies.comp:51-54) */
static inline v3 colmul(const real* m, v3 v) {
    return mk((m[0] * v.x + m[3] * v.y) + m[6] * v.z, (m[1] * v.x + m[4] * v.y) + m[7] * v.z,
              (m[2] * v.x + m[5] * v.y) + m[8] * v.z);
}
static inline void st_state(real* q, real* qd, int64_t b, v3 p, q4 r, v3 v, v3 w) {
    q[b * 8 + 0] = p.x; q[b * 8 + 1] = p.y; q[b * 8 + 2] = p.z; q[b * 8 + 3] = RF(0.0);
    q[b * 8 + 4] = r.x; q[b * 8 + 5] = r.y; q[b * 8 + 6] = r.z; q[b * 8 + 7] = r.w;
    qd[b * 8 + 0] = v.x; qd[b * 8 + 1] = v.y; qd[b * 8 + 2] = v.z; qd[b * 8 + 3] = RF(0.0);
    qd[b * 8 + 4] = w.x; qd[b * 8 + 5] = w.y; qd[b * 8 + 6] = w.z; qd[b * 8 + 7] = RF(0.0);
}

/* integrate_bodies.comp:75-130 for body b (body forces are zero) */
static void integrate_body(const or_solver* s, int64_t b, real dt, const real* q, const real* qd, real* qo,
                           real* qdo) {
    if (s->body_flags[b] & 2) { /* KINEMATIC */
        memcpy(qo + b * 8, q + b * 8, 8 * sizeof(real));
        memcpy(qdo + b * 8, qd + b * 8, 8 * sizeof(real));
        return;
    }
    v3 x0, w0, v0;
    q4 r0;
    body_state(q, b, &x0, &r0);
    v0 = mk(qd[b * 8], qd[b * 8 + 1], qd[b * 8 + 2]);
    w0 = mk(qd[b * 8 + 4], qd[b * 8 + 5], qd[b * 8 + 6]);
    v3 f0 = mk(RF(0.0), RF(0.0), RF(0.0)), t0 = f0;
    v3 com = ld3(s->body_com, b);
    real inv_mass = s->body_invm[b];
    v3 g = mk((real)s->cfg.gravity[0], (real)s->cfg.gravity[1], (real)s->cfg.gravity[2]);
    v3 x_com = vadd(x0, wq_rot(r0, com));
    real m_scale = inv_mass != RF(0.0) ? RF(1.0) : RF(0.0);
    v3 v1 = vadd(v0, vmuls(vadd(vmuls(f0, inv_mass), vmuls(g, m_scale)), dt));
    v3 x1 = vadd(x_com, vmuls(v1, dt));
    v3 wb = wq_rot_inv(r0, w0);
    v3 Iwb = colmul(&s->body_I[b * 9], wb);
    v3 tb = vsub(wq_rot_inv(r0, t0), vcross(wb, Iwb));
    v3 dwb = vmuls(colmul(&s->body_invI[b * 9], tb), dt);
    v3 w1 = wq_rot(r0, vadd(wb, dwb));
    q4 wq;
    wq.x = w1.x; wq.y = w1.y; wq.z = w1.z; wq.w = RF(0.0);
    q4 r1 = q_normalize(q_axpy(r0, wq_mul(wq, r0), RF(0.5) * dt));
    w1 = vmuls(w1, RF(1.0) - (real)s->bp.angular_damping * dt);
    st_state(qo, qdo, b, vsub(x1, wq_rot(r1, com)), r1, v1, w1);
}

/* apply_body_deltas.comp:58-119 for body b with the 6-float delta d (lin, ang) */
static void apply_body_delta(const or_solver* s, int64_t b, real dt, const real* q, const real* qd, const real* d,
                             real inv_weight, int use_weights, real* qo, real* qdo) {
    real inv_m = s->body_invm[b];
    if (inv_m == RF(0.0)) {
        memcpy(qo + b * 8, q + b * 8, 8 * sizeof(real));
        memcpy(qdo + b * 8, qd + b * 8, 8 * sizeof(real));
        return;
    }
    v3 pos0, v0, w0;
    q4 quat0;
    body_state(q, b, &pos0, &quat0);
    v0 = mk(qd[b * 8], qd[b * 8 + 1], qd[b * 8 + 2]);
    w0 = mk(qd[b * 8 + 4], qd[b * 8 + 5], qd[b * 8 + 6]);
    const real* I9 = &s->body_I[b * 9];
    const real* Iinv9 = &s->body_invI[b * 9];
    v3 com = ld3(s->body_com, b);
    v3 dp = mk(d[0], d[1], d[2]), dq = mk(d[3], d[4], d[5]);
    real weight = RF(1.0);
    if (use_weights) {
        if (inv_weight > RF(0.0)) weight = RF(1.0) / inv_weight;
    }
    dp = vmuls(dp, inv_m * weight);
    v3 dq_w = vmuls(dq, weight);
    v3 wb = wq_rot_inv(quat0, w0);
    v3 dwb = colmul(Iinv9, wq_rot_inv(quat0, dq_w));
    v3 tb = vadd(vcross(dwb, colmul(I9, vadd(wb, dwb))), vcross(wb, colmul(I9, dwb)));
    v3 dw1 = wq_rot(quat0, vsub(dwb, vmuls(colmul(Iinv9, tb), dt)));
    q4 dq4;
    dq4.x = dw1.x * dt; dq4.y = dw1.y * dt; dq4.z = dw1.z * dt; dq4.w = RF(0.0);
    q4 quat1 = q_normalize(q_axpy(quat0, wq_mul(dq4, quat0), RF(0.5)));
    v3 x_com = vadd(pos0, wq_rot(quat0, com));
    v3 p1 = vadd(x_com, vmuls(dp, dt));
    p1 = vsub(p1, wq_rot(quat1, com));
    v3 v1 = vadd(v0, dp), w1 = vadd(w0, dw1);
    if (vlength(v1) < RF(1e-4)) v1 = mk(RF(0.0), RF(0.0), RF(0.0));
    if (vlength(w1) < RF(1e-4)) w1 = mk(RF(0.0), RF(0.0), RF(0.0));
    st_state(qo, qdo, b, p1, quat1, v1, w1);
}

/* compute_contact_constraint_delta, solve_body_contact_positions.comp:63-83 */
static real contact_constraint_delta(real err, q4 qa, q4 qb, real m_inv_a, real m_inv_b, const real* ia,
                                     const real* ib, v3 lin_a, v3 lin_b, v3 ang_a, v3 ang_b, real relax, real dt) {
    real denom = RF(0.0);
    denom += vdot(lin_a, lin_a) * m_inv_a;
    denom += vdot(lin_b, lin_b) * m_inv_b;
    v3 ra = wq_rot_inv(qa, ang_a), rb = wq_rot_inv(qb, ang_b);
    denom += vdot(ra, colmul(ia, ra));
    denom += vdot(rb, colmul(ib, rb));
    real dl = -err;
    if (denom > RF(0.0)) dl /= dt * denom;
    return dl * relax;
}

typedef struct { v3 lin_a, ang_a, lin_b, ang_b; } rc_delta;

/* solve_body_contact_positions.comp:97-265 for one contact of shape_a (the
 * contact-impulse debug output is not kept). Returns 0 when it is skipped. */
static int body_contact(const or_solver* s, const real* q, const real* qd, int32_t shape_a, const or_rcontact* c,
                        real dt, rc_delta* o) {
    static const real zero9[9] = {0};
    int32_t shape_b = c->shape1;
    if (shape_a == shape_b) return 0;
    int32_t body_a = shape_a >= 0 ? s->shape_body[shape_a] : -1;
    int32_t body_b = shape_b >= 0 ? s->shape_body[shape_b] : -1;
    if (body_a == body_b) return 0;
    v3 pos_a = mk(RF(0.0), RF(0.0), RF(0.0)), pos_b = pos_a;
    q4 quat_a = {RF(0.0), RF(0.0), RF(0.0), RF(1.0)}, quat_b = quat_a;
    if (body_a >= 0) body_state(q, body_a, &pos_a, &quat_a);
    if (body_b >= 0) body_state(q, body_b, &pos_b, &quat_b);
    v3 bx_a = vadd(wq_rot(quat_a, c->p0), pos_a);
    v3 bx_b = vadd(wq_rot(quat_b, c->p1), pos_b);
    v3 n = c->n;
    real d = vdot(n, vsub(bx_b, bx_a)) - (c->th0 + c->th1);
    if (d >= RF(0.0)) return 0;
    real m_inv_a = RF(0.0), m_inv_b = RF(0.0);
    const real *ia = zero9, *ib = zero9;
    v3 com_a = mk(RF(0.0), RF(0.0), RF(0.0)), com_b = com_a, omega_a = com_a, omega_b = com_a;
    if (body_a >= 0) {
        m_inv_a = s->body_invm[body_a];
        ia = &s->body_invI[body_a * 9];
        com_a = ld3(s->body_com, body_a);
        omega_a = mk(qd[body_a * 8 + 4], qd[body_a * 8 + 5], qd[body_a * 8 + 6]);
    }
    if (body_b >= 0) {
        m_inv_b = s->body_invm[body_b];
        ib = &s->body_invI[body_b * 9];
        com_b = ld3(s->body_com, body_b);
        omega_b = mk(qd[body_b * 8 + 4], qd[body_b * 8 + 5], qd[body_b * 8 + 6]);
    }
    /* material averages (:159-178): every shape carries shape_material_mu and the
     * torsional / rolling coefficients of the body parameters */
    int nz = 0;
    real mu = RF(0.0), mu_t = RF(0.0), mu_r = RF(0.0);
    if (shape_a >= 0) { nz += 1; mu += s->shape_mu[shape_a]; mu_t += (real)s->bp.rigid_mu_torsional; mu_r += (real)s->bp.rigid_mu_rolling; }
    if (shape_b >= 0) { nz += 1; mu += s->shape_mu[shape_b]; mu_t += (real)s->bp.rigid_mu_torsional; mu_r += (real)s->bp.rigid_mu_rolling; }
    if (nz > 0) {
        mu /= (real)nz;
        mu_t /= (real)nz;
        mu_r /= (real)nz;
    }
    v3 r_a = vsub(bx_a, vadd(wq_rot(quat_a, com_a), pos_a));
    v3 r_b = vsub(bx_b, vadd(wq_rot(quat_b, com_b), pos_b));
    v3 angular_a = vneg(vcross(r_a, n));
    v3 angular_b = vcross(r_b, n);
    real relax = (real)s->bp.rigid_contact_relaxation;
    real lambda_n = contact_constraint_delta(d, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, vneg(n), n, angular_a,
                                             angular_b, relax, dt);
    v3 lin_da = vmuls(vneg(n), lambda_n), lin_db = vmuls(n, lambda_n);
    v3 ang_da = vmuls(angular_a, lambda_n), ang_db = vmuls(angular_b, lambda_n);
    if (mu > RF(0.0)) {
        v3 sbx_a = vadd(wq_rot(quat_a, vadd(c->p0, c->off0)), pos_a);
        v3 sbx_b = vadd(wq_rot(quat_b, vadd(c->p1, c->off1)), pos_b);
        v3 delta = vsub(sbx_b, sbx_a);
        v3 fdel = vsub(delta, vmuls(n, vdot(n, delta)));
        v3 fr_a = vsub(sbx_a, vadd(wq_rot(quat_a, com_a), pos_a));
        v3 fr_b = vsub(sbx_b, vadd(wq_rot(quat_b, com_b), pos_b));
        v3 rel = mk(RF(0.0), RF(0.0), RF(0.0));
        if (body_a >= 0 && (s->body_flags[body_a] & 2)) {
            v3 va = vadd(mk(qd[body_a * 8], qd[body_a * 8 + 1], qd[body_a * 8 + 2]), vcross(omega_a, fr_a));
            rel = vsub(rel, vsub(va, vmuls(n, vdot(n, va))));
        }
        if (body_b >= 0 && (s->body_flags[body_b] & 2)) {
            v3 vb = vadd(mk(qd[body_b * 8], qd[body_b * 8 + 1], qd[body_b * 8 + 2]), vcross(omega_b, fr_b));
            rel = vadd(rel, vsub(vb, vmuls(n, vdot(n, vb))));
        }
        fdel = vadd(fdel, vmuls(rel, dt));
        real err = vlength(fdel);
        if (err > RF(0.0)) {
            v3 perp = vnormalize(fdel);
            v3 angular_a_fr = vneg(vcross(fr_a, perp));
            v3 angular_b_fr = vcross(fr_b, perp);
            real lambda_fr = contact_constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, vneg(perp), perp,
                                                      angular_a_fr, angular_b_fr, relax, dt);
            lambda_fr = gmax(lambda_fr, -lambda_n * mu);
            lin_da = vsub(lin_da, vmuls(perp, lambda_fr));
            lin_db = vadd(lin_db, vmuls(perp, lambda_fr));
            ang_da = vadd(ang_da, vmuls(angular_a_fr, lambda_fr));
            ang_db = vadd(ang_db, vmuls(angular_b_fr, lambda_fr));
        }
    }
    v3 delta_omega = vsub(omega_b, omega_a);
    v3 zero = mk(RF(0.0), RF(0.0), RF(0.0));
    if (mu_t > RF(0.0)) {
        real err = vdot(delta_omega, n) * dt;
        if (R_FABS(err) > RF(0.0)) {
            real lt = contact_constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, zero, zero, vneg(n), n,
                                               relax, dt);
            lt = gclamp(lt, -lambda_n * mu_t, lambda_n * mu_t);
            ang_da = vsub(ang_da, vmuls(n, lt));
            ang_db = vadd(ang_db, vmuls(n, lt));
        }
    }
    if (mu_r > RF(0.0)) {
        delta_omega = vsub(delta_omega, vmuls(n, vdot(n, delta_omega)));
        real err = vlength(delta_omega) * dt;
        if (err > RF(0.0)) {
            v3 roll_n = vnormalize(delta_omega);
            real lr = contact_constraint_delta(err, quat_a, quat_b, m_inv_a, m_inv_b, ia, ib, zero, zero,
                                               vneg(roll_n), roll_n, relax, dt);
            lr = gmax(lr, -lambda_n * mu_r);
            ang_da = vsub(ang_da, vmuls(roll_n, lr));
            ang_db = vadd(ang_db, vmuls(roll_n, lr));
        }
    }
    o->lin_a = lin_da;
    o->ang_a = ang_da;
    o->lin_b = lin_db;
    o->ang_b = ang_db;
    return 1;
}

static int64_t mesh_vert_off(const or_solver* s, int64_t m) {
    int64_t o = 0;
    for (int64_t c = 0; c < m; c++) o += s->meshes[c].nv;
    return o;
}

/* Rigid contact generation (no reference counterpart: nothing in the reference
 * generates the contacts solve_body_contact_positions.comp reads). Every vertex of
 * a dynamic body's mesh is tested against the ground plane and, with the particle
 * closest-point query of generate_mesh_contacts.comp at radius 0, against every
 * other mesh; up to RC_CAP contacts per vertex, plane first, then meshes in index
 * order. Uses the body states at the start of the substep. */
static void rigid_collide(or_solver* s) {
    real margin = (real)s->bp.rigid_contact_margin;
    real alt = (real)s->cfg.ground_plane_altitude;
    int ovf = 0;
    for (int64_t a = 0; a < s->nmesh; a++) {
        if (!posed(s, a)) continue;
        v3 pos_a;
        q4 rot_a;
        body_state(s->body_q, a, &pos_a, &rot_a);
        real th0 = (real)s->meshes[a].margin;
        int64_t vo = mesh_vert_off(s, a);
        for (int64_t v = 0; v < s->meshes[a].nv; v++) {
            int64_t gv = vo + v;
            v3 V = ld3f(s->all_verts, gv);
            v3 P = vadd(pos_a, quat_rotate(rot_a, V));
            int cnt = 0;
            or_rcontact* out = &s->rc[gv * RC_CAP];
            if (s->cfg.has_ground_plane) {
                real dist = P.z - alt;
                if (dist < margin) {
                    or_rcontact* c = &out[cnt++];
                    c->shape1 = 0;
                    c->n = mk(RF(0.0), RF(0.0), RF(-1.0));
                    c->p0 = V;
                    c->p1 = mk(P.x, P.y, alt);
                    c->th0 = th0;
                    c->th1 = RF(0.0);
                    c->off0 = quat_rotate_inv(rot_a, vmuls(c->n, th0));
                    c->off1 = vmuls(c->n, -c->th1);
                }
            }
            for (int64_t m = 0; m < s->nmesh; m++) {
                if (m == a) continue;
                v3 Q = P, bpos, bvel, nrm, pos_m;
                q4 rot_m;
                int pz = posed(s, m);
                if (pz) {
                    body_state(s->body_q, m, &pos_m, &rot_m);
                    Q = quat_rotate_inv(rot_m, vsub(P, pos_m));
                }
                if (!mesh_query(s, m, Q, RF(0.0), margin, &bpos, &bvel, &nrm, &ovf)) continue;
                if (cnt >= RC_CAP) {
                    s->rc_overflow++;
                    continue;
                }
                or_rcontact* c = &out[cnt++];
                real th1 = (real)s->meshes[m].margin;
                c->shape1 = (int32_t)m + 1;
                c->n = vneg(pz ? quat_rotate(rot_m, nrm) : nrm);
                c->p0 = V;
                c->p1 = bpos;
                c->th0 = th0;
                c->th1 = th1;
                c->off0 = quat_rotate_inv(rot_a, vmuls(c->n, th0));
                c->off1 = pz ? quat_rotate_inv(rot_m, vmuls(c->n, -th1)) : vmuls(c->n, -th1);
            }
            s->rc_cnt[gv] = cnt;
        }
    }
    if (ovf) fprintf(stderr, "oracle: BVH traversal stack overflow (push dropped)\n");
}

/* One body pass of an iteration: particle-contact body deltas (summed per body in
 * contact-slot order) applied with the number of those contacts as constraint
 * weight (apply_body_deltas.comp:85-89; a switch turns it off), then the rigid
 * contacts solved on that state and applied with their own count as weight. */
static void bodies_iterate(or_solver* s, real dt) {
    int64_t nb = s->nbody;
    real* d6 = xcalloc((size_t)nb * 6, sizeof(real));
    real* wc = xcalloc((size_t)nb, sizeof(real));
    int64_t count = s->ccount_raw < s->cmax ? s->ccount_raw : s->cmax;
    for (int64_t t = 0; t < count; t++) {
        if (!s->bvalid[t]) continue;
        int32_t b = s->shape_body[s->cshape[t]];
        for (int k = 0; k < 6; k++) d6[b * 6 + k] += s->bdel[t * 6 + k];
        wc[b] += RF(1.0);
    }
    for (int64_t b = 0; b < nb; b++)
        apply_body_delta(s, b, dt, s->body_q, s->body_qd, &d6[b * 6], wc[b], s->bp.particle_contact_con_weighting,
                         s->body_qm, s->body_qdm);
    memset(wc, 0, sizeof(real) * (size_t)nb);
    memset(d6, 0, sizeof(real) * 6 * (size_t)nb);
    for (int64_t x = 0; x < nb; x++) {
        if (!posed(s, x)) continue;
        v3 lin = mk(RF(0.0), RF(0.0), RF(0.0)), ang = lin;
        real cnt = RF(0.0);
        rc_delta o;
        int64_t vo = mesh_vert_off(s, x);
        for (int64_t v = 0; v < s->meshes[x].nv; v++) /* x as shape0: its own vertices */
            for (int j = 0; j < s->rc_cnt[vo + v]; j++)
                if (body_contact(s, s->body_qm, s->body_qdm, (int32_t)x + 1, &s->rc[(vo + v) * RC_CAP + j], dt, &o)) {
                    lin = vadd(lin, o.lin_a);
                    ang = vadd(ang, o.ang_a);
                    cnt += RF(1.0);
                }
        for (int64_t a = 0; a < nb; a++) { /* x as shape1: other bodies' vertices on x's mesh */
            if (a == x || !posed(s, a)) continue;
            int64_t ao = mesh_vert_off(s, a);
            for (int64_t v = 0; v < s->meshes[a].nv; v++)
                for (int j = 0; j < s->rc_cnt[ao + v]; j++) {
                    const or_rcontact* c = &s->rc[(ao + v) * RC_CAP + j];
                    if (c->shape1 != (int32_t)x + 1) continue;
                    if (body_contact(s, s->body_qm, s->body_qdm, (int32_t)a + 1, c, dt, &o)) {
                        lin = vadd(lin, o.lin_b);
                        ang = vadd(ang, o.ang_b);
                        cnt += RF(1.0);
                    }
                }
        }
        d6[x * 6 + 0] = lin.x; d6[x * 6 + 1] = lin.y; d6[x * 6 + 2] = lin.z;
        d6[x * 6 + 3] = ang.x; d6[x * 6 + 4] = ang.y; d6[x * 6 + 5] = ang.z;
        wc[x] = cnt;
    }
    for (int64_t b = 0; b < nb; b++)
        apply_body_delta(s, b, dt, s->body_qm, s->body_qdm, &d6[b * 6], wc[b], s->bp.rigid_contact_con_weighting,
                         s->body_q, s->body_qd);
    free(d6);
    free(wc);
}

static void iterate(or_solver* s, real dt, int iterations, real inv) { /* scene.cpp:934-980 */
    int64_t n = s->n;
    int64_t count = s->ccount_raw < s->cmax ? s->ccount_raw : s->cmax;
    for (int it = 0; it < iterations; it++) {
        memset(s->delta, 0, sizeof(real) * 3 * (size_t)n);
        if (s->dyn_any) memset(s->bvalid, 0, (size_t)s->cmax);
        for (int64_t t = 0; t < count; t++) shape_contact(s, t, s->x, s->v, dt);
#ifdef _OPENMP
#pragma omp parallel for OMP_THREADS schedule(static, 256)
#endif
        for (int64_t t = 0; t < n; t++) pp_contact(s, t, s->x, s->v, dt, inv);
        apply_deltas(s, s->x, s->v, dt);
        real* t0 = s->x; s->x = s->xo; s->xo = t0;
        real* t1 = s->v; s->v = s->vo; s->vo = t1;
        if (s->dyn_any) bodies_iterate(s, dt);
    }
}

static void restitution(or_solver* s) { /* scene.cpp:983-989 */
    if (!s->cfg.enable_restitution) return;
    int64_t count = s->ccount_raw < s->cmax ? s->ccount_raw : s->cmax;
    memcpy(s->vsnap, s->v, sizeof(real) * 3 * (size_t)s->n);
    for (int64_t t = 0; t < count; t++) restitution_contact(s, t);
}

/* ------------------------------------------------------------------------- */
/* Differentiable rollout: forward trajectory and hand-written adjoint          */
/* ------------------------------------------------------------------------- */

/* pair_backward: exact derivative of one particle-particle term of
 * solve_particle_particle_contacts.comp:159-177 (pair_d = diff / (w_i + w_j)) for the
 * upstream gradient G of pair_d; the contact set and the max() branch are fixed. */
static void pair_backward(v3 raw, v3 vrel, real ri, real rj, real wi, real wj, real k_mu, real dt, v3 G, v3* g_u,
                          v3* g_vrel, real* g_w, real* g_kmu, v3* pair_d) {
    /* forward values, computed as the forward computes them (branch decisions must agree) */
    real d = exact_length(raw);
    real err = d - ri - rj;
    real denom = wi + wj;
    v3 nn = exact_div(raw, d);
    real vn = exact_dot(nn, vrel);
    v3 vt = mk(R_FMA(vn, -nn.x, vrel.x), R_FMA(vn, -nn.y, vrel.y), R_FMA(vn, -nn.z, vrel.z));
    real vt_len = exact_length(vt);
    real a = k_mu * err, b = -vt_len * dt;
    int branch_a = !(a < b);
    real lf = branch_a ? a : b;
    v3 vt_dir = vt_len > RF(0.0) ? exact_div(vt, vt_len) : mk(RF(0.0), RF(0.0), RF(0.0));
    v3 p2 = vmuls(nn, err);
    v3 diff = mk(R_FMA(vt_dir.x, lf, -p2.x), R_FMA(vt_dir.y, lf, -p2.y), R_FMA(vt_dir.z, lf, -p2.z));
    *pair_d = exact_div(diff, denom);
    /* reverse mode */
    v3 g_diff = vmuls(G, RF(1.0) / denom);
    *g_w = -vdot(G, diff) / (denom * denom);
    v3 g_vt_dir = vmuls(g_diff, lf);
    real g_lf = vdot(g_diff, vt_dir);
    v3 g_nn = vmuls(g_diff, -err);
    real g_err = -vdot(g_diff, nn);
    real g_vt_len = RF(0.0);
    if (branch_a) {
        g_err += k_mu * g_lf;
        *g_kmu += err * g_lf;
    } else {
        g_vt_len = -dt * g_lf;
    }
    v3 g_vt = mk(RF(0.0), RF(0.0), RF(0.0));
    if (vt_len > RF(0.0))
        g_vt = vadd(vmuls(vsub(g_vt_dir, vmuls(vt_dir, vdot(vt_dir, g_vt_dir))), RF(1.0) / vt_len),
                    vmuls(vt_dir, g_vt_len));
    v3 gv = g_vt;
    real g_vn = -vdot(g_vt, nn);
    g_nn = vadd(g_nn, vmuls(g_vt, -vn));
    g_nn = vadd(g_nn, vmuls(vrel, g_vn));
    gv = vadd(gv, vmuls(nn, g_vn));
    *g_vrel = gv;
    *g_u = vadd(vmuls(vsub(g_nn, vmuls(nn, vdot(nn, g_nn))), RF(1.0) / d), vmuls(nn, g_err));
}

/* The particle-particle term of pair (i, j) with the forward's filters
 * (solve_particle_particle_contacts.comp:145-157); returns 0 when it is skipped. */
static int pair_term(const or_solver* s, int32_t i, int32_t j, const real* X, real R, v3* raw_out) {
    v3 raw = vsub(ld3(X, i), ld3(X, j));
    if (R_FABS(raw.x) > R || R_FABS(raw.y) > R || R_FABS(raw.z) > R) return 0;
    real d = exact_length(raw);
    real err = d - s->r[i] - s->r[j];
    if (err > (real)s->cfg.particle_cohesion || d <= RF(0.0)) return 0;
    if (s->w[i] + s->w[j] <= RF(0.0)) return 0;
    *raw_out = raw;
    return 1;
}

static or_traj* traj_of(or_solver* s) { return &s->traj; }

int or_rollout(or_solver* s, float dt, int substeps, int iterations, int frames) {
    if (!s->finalized) or_finalize_meshes(s);
    if (s->nmesh > 0 || iterations != 1) return -1;
    or_traj* T = traj_of(s);
    free(T->x);
    free(T->v);
    T->steps = (int64_t)substeps * frames;
    size_t n3 = (size_t)s->n * 3;
    T->x = xcalloc((size_t)(T->steps + 1) * n3, sizeof(real));
    T->v = xcalloc((size_t)(T->steps + 1) * n3, sizeof(real));
    float sdt_f = dt / (float)substeps;
    float inv_f = 1.0f / s->cfg.search_radius;
    T->sdt = (real)sdt_f;
    T->inv = (real)inv_f;
    T->clamped = 0;
    int64_t t = 0;
    for (int f = 0; f < frames; f++)
        for (int sub = 0; sub < substeps; sub++, t++) {
            memcpy(T->x + (size_t)t * n3, s->x, n3 * sizeof(real));
            memcpy(T->v + (size_t)t * n3, s->v, n3 * sizeof(real));
            collide(s);
            integrate(s, T->sdt);
            for (int64_t i = 0; i < s->n; i++)
                if (vlength(ld3(s->v, i)) > (real)s->cfg.particle_v_max) T->clamped = 1;
            build_grid(s, T->inv);
            iterate(s, T->sdt, 1, T->inv);
            restitution(s);
            for (int64_t i = 0; i < s->n; i++)
                if (vlength(ld3(s->v, i)) > RF(0.5) * (real)s->cfg.particle_v_max) T->clamped = 1;
        }
    memcpy(T->x + (size_t)t * n3, s->x, n3 * sizeof(real));
    memcpy(T->v + (size_t)t * n3, s->v, n3 * sizeof(real));
    return 0;
}

int or_rollout_backward(or_solver* s, const float* gx_final, const float* gv_final, double* gx0_out,
                        double* gv0_out, double* gw_out, double* params) {
    or_traj* T = traj_of(s);
    if (!T->x) return -1;
    if (T->clamped) return -2;
    int64_t n = s->n;
    size_t n3 = (size_t)n * 3;
    real dt = T->sdt, inv = T->inv;
    real relax = (real)s->cfg.soft_contact_relaxation;
    real ka = (real)s->cfg.particle_adhesion;
    real e = (real)s->cfg.soft_contact_restitution;
    real mu_plane = RF(0.5) * ((real)s->cfg.soft_contact_mu + s->shape_mu[0]);
    real k_mu = (real)s->cfg.particle_mu;
    real* Gx = xcalloc(n3, sizeof(real));
    real* Gv = xcalloc(n3, sizeof(real));
    real* gxp = xcalloc(n3, sizeof(real));
    real* gvp = xcalloc(n3, sizeof(real));
    real* gx0 = xcalloc(n3, sizeof(real));
    real* gv0 = xcalloc(n3, sizeof(real));
    real* gw = xcalloc((size_t)n, sizeof(real));
    real g_mu = RF(0.0), g_kmu = RF(0.0), g_e = RF(0.0);
    for (size_t k = 0; k < n3; k++) {
        Gx[k] = (real)gx_final[k];
        Gv[k] = gv_final ? (real)gv_final[k] : RF(0.0);
    }
    for (int64_t t = T->steps - 1; t >= 0; t--) {
        /* replay the forward's intermediates of substep t */
        memcpy(s->x, T->x + (size_t)t * n3, n3 * sizeof(real));
        memcpy(s->v, T->v + (size_t)t * n3, n3 * sizeof(real));
        collide(s);
        integrate(s, dt); /* s->x, s->v = predicted; s->x0, s->v0 = start of the substep */
        build_grid(s, inv);
        memset(gx0, 0, n3 * sizeof(real));
        memset(gv0, 0, n3 * sizeof(real));
        memset(gvp, 0, n3 * sizeof(real));
        int64_t count = s->ccount_raw < s->cmax ? s->ccount_raw : s->cmax;
        real* gv1 = Gv; /* restitution: v_final.z = v1.z + (-v1.z + max(-e v0.z, 0)) */
        if (s->cfg.enable_restitution) {
            for (int64_t c = 0; c < count; c++) {
                int32_t i = s->cpart[c];
                v3 x0 = ld3(s->x0, i), v0 = ld3(s->v0, i);
                v3 bx = ld3(s->cbpos, c);
                real cc = (x0.z - bx.z) - s->r[i];
                if (cc > ka) continue;
                real rel_old = v0.z;
                if (!(rel_old < RF(0.0))) continue;
                real g_rt = gv1[i * 3 + 2];
                gv1[i * 3 + 2] = RF(0.0);
                if ((-e) * rel_old > RF(0.0)) {
                    gv0[i * 3 + 2] += g_rt * (-e);
                    g_e += g_rt * (-rel_old);
                }
            }
        }
        /* apply: x1 = xp + delta, v1 = (x1 - x0) / dt */
        for (size_t k = 0; k < n3; k++) {
            real gx1 = Gx[k] + gv1[k] / dt;
            gx0[k] -= gv1[k] / dt;
            gxp[k] = gx1; /* also dL/d delta */
        }
        real* gdelta = xcalloc(n3, sizeof(real));
        memcpy(gdelta, gxp, n3 * sizeof(real));
        /* plane contacts (solve_particle_shape_contacts.comp with w2 = 0) */
        for (int64_t c = 0; c < count; c++) {
            int32_t i = s->cpart[c];
            v3 xp = ld3(s->x, i), vp = ld3(s->v, i);
            v3 bx = ld3(s->cbpos, c);
            real cc = (xp.z - bx.z) - s->r[i];
            if (cc > ka) continue;
            v3 vt = mk(vp.x, vp.y, RF(0.0));
            real vt_len = exact_length(vt);
            real a = mu_plane * cc, b = -vt_len * dt;
            int branch_a = !(a < b);
            real lf = branch_a ? a : b;
            v3 vt_dir = vt_len > RF(0.0) ? exact_div(vt, vt_len) : mk(RF(0.0), RF(0.0), RF(0.0));
            v3 g_diff = vmuls(ld3(gdelta, i), relax);
            v3 g_vt_dir = vmuls(g_diff, lf);
            real g_lf = vdot(g_diff, vt_dir);
            real g_c = -g_diff.z, g_vt_len = RF(0.0);
            if (branch_a) {
                g_c += mu_plane * g_lf;
                g_mu += cc * g_lf;
            } else {
                g_vt_len = -dt * g_lf;
            }
            if (vt_len > RF(0.0)) {
                v3 g_vt = vadd(vmuls(vsub(g_vt_dir, vmuls(vt_dir, vdot(vt_dir, g_vt_dir))), RF(1.0) / vt_len),
                               vmuls(vt_dir, g_vt_len));
                gvp[i * 3 + 0] += g_vt.x;
                gvp[i * 3 + 1] += g_vt.y;
            }
            gxp[i * 3 + 2] += g_c;
        }
        /* particle-particle: total_i = w_i * relax * sum_j pair_d_ij */
        real R_add = (real)s->cfg.particle_max_radius + (real)s->cfg.particle_cohesion;
        for (int64_t tid = 0; tid < n; tid++) {
            int32_t i = (int32_t)s->sids[tid];
            v3 x = ld3(s->x, i);
            real R = s->r[i] + R_add;
            v3 Gi = ld3(gdelta, i);
            v3 gacc = vmuls(Gi, s->w[i] * relax);
            v3 acc = mk(RF(0.0), RF(0.0), RF(0.0));
            int32_t xs = f2i(R_FLOOR((x.x - R) * inv)), ys = f2i(R_FLOOR((x.y - R) * inv)),
                    zs = f2i(R_FLOOR((x.z - R) * inv));
            int32_t xe = f2i(R_FLOOR((x.x + R) * inv)), ye = f2i(R_FLOOR((x.y + R) * inv)),
                    ze = f2i(R_FLOOR((x.z + R) * inv));
            if (xe > xs + GRID_DIM - 1) xe = xs + GRID_DIM - 1;
            if (ye > ys + GRID_DIM - 1) ye = ys + GRID_DIM - 1;
            if (ze > zs + GRID_DIM - 1) ze = zs + GRID_DIM - 1;
            for (int32_t cz = zs; cz <= ze; cz++)
                for (int32_t cy = ys; cy <= ye; cy++)
                    for (int32_t cx = xs; cx <= xe; cx++) {
                        int32_t cell = cell_index(cx, cy, cz);
                        for (int32_t k = s->cstart[cell]; k < s->cend[cell]; k++) {
                            int32_t j = (int32_t)s->sids[k];
                            v3 raw;
                            if (j == i || !pair_term(s, i, j, s->x, R, &raw)) continue;
                            v3 vrel = vsub(ld3(s->v, i), ld3(s->v, j));
                            v3 g_u, g_vrel, pd;
                            real g_den;
                            pair_backward(raw, vrel, s->r[i], s->r[j], s->w[i], s->w[j], k_mu, dt, gacc, &g_u, &g_vrel,
                                          &g_den, &g_kmu, &pd);
                            acc = vadd(acc, pd);
                            for (int a = 0; a < 3; a++) {
                                real gu = a == 0 ? g_u.x : (a == 1 ? g_u.y : g_u.z);
                                real gvr = a == 0 ? g_vrel.x : (a == 1 ? g_vrel.y : g_vrel.z);
                                gxp[i * 3 + a] += gu;
                                gxp[j * 3 + a] -= gu;
                                gvp[i * 3 + a] += gvr;
                                gvp[j * 3 + a] -= gvr;
                            }
                            gw[i] += g_den;
                            gw[j] += g_den;
                        }
                    }
            gw[i] += vdot(Gi, acc) * relax;
        }
        free(gdelta);
        /* integrate: xp = x0 + vp dt, vp = v0 + g dt [w > 0] */
        for (size_t k = 0; k < n3; k++) {
            gvp[k] += gxp[k] * dt;
            Gx[k] = gx0[k] + gxp[k];
            Gv[k] = gv0[k] + gvp[k];
        }
    }
    for (size_t k = 0; k < n3; k++) {
        if (gx0_out) gx0_out[k] = (double)Gx[k];
        if (gv0_out) gv0_out[k] = (double)Gv[k];
    }
    for (int64_t i = 0; i < n; i++)
        if (gw_out) gw_out[i] = (double)gw[i];
    if (params) {
        params[0] = (double)(RF(0.5) * g_mu);
        params[1] = (double)(RF(0.5) * g_mu);
        params[2] = (double)g_kmu;
        params[3] = (double)g_e;
    }
    /* leave the solver at the final state of the rollout */
    memcpy(s->x, T->x + (size_t)T->steps * n3, n3 * sizeof(real));
    memcpy(s->v, T->v + (size_t)T->steps * n3, n3 * sizeof(real));
    free(Gx); free(Gv); free(gxp); free(gvp); free(gx0); free(gv0); free(gw);
    return 0;
}

int or_step(or_solver* s, float dt, int substeps, int iterations) { /* scene.cpp:698-1092 */
    if (!s->finalized) or_finalize_meshes(s);
    float sdt_f = dt / (float)substeps;
    float inv_f = 1.0f / s->cfg.search_radius;
    real sdt = (real)sdt_f, inv = (real)inv_f;
    for (int sub = 0; sub < substeps; sub++) {
        collide(s);
        if (s->dyn_any) rigid_collide(s);
        integrate(s, sdt);
        if (s->dyn_any) {
            memcpy(s->body_qp, s->body_q, sizeof(real) * 8 * (size_t)s->nbody);
            memcpy(s->body_qdp, s->body_qd, sizeof(real) * 8 * (size_t)s->nbody);
            for (int64_t b = 0; b < s->nbody; b++)
                integrate_body(s, b, sdt, s->body_qp, s->body_qdp, s->body_q, s->body_qd);
        }
        build_grid(s, inv);
        iterate(s, sdt, iterations, inv);
        restitution(s);
    }
    return 0;
}

int or_collide_only(or_solver* s) { /* scene.cpp:1229-1245 */
    if (!s->finalized) or_finalize_meshes(s);
    collide(s);
    return 0;
}

int or_set_contact_data(or_solver* s, const int32_t* part, const int32_t* shape, const float* bpos,
                        const float* nrm, int64_t count) { /* scene.cpp:1304-1315 */
    s->ccount_raw = count;
    int64_t m = count < s->cmax ? count : s->cmax;
    for (int64_t t = 0; t < m; t++) {
        s->cpart[t] = part[t];
        s->cshape[t] = shape[t];
        st3(s->cbpos, t, ld3f(bpos, t));
        st3(s->cnorm, t, ld3f(nrm, t));
        st3(s->cbvel, t, mk(RF(0.0), RF(0.0), RF(0.0)));
    }
    return 0;
}

int or_step_solve_only(or_solver* s, float dt, int substeps, int iterations) { /* scene.cpp:1094-1227 */
    if (!s->finalized) or_finalize_meshes(s);
    float sdt_f = dt / (float)substeps;
    float inv_f = 1.0f / s->cfg.search_radius;
    real sdt = (real)sdt_f, inv = (real)inv_f;
    for (int sub = 0; sub < substeps; sub++) {
        integrate(s, sdt);
        build_grid(s, inv);
        iterate(s, sdt, iterations, inv);
        restitution(s);
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* Getters                                                                     */
/* ------------------------------------------------------------------------- */
void or_get_positions(const or_solver* s, float* out) {
    for (int64_t i = 0; i < s->n * 3; i++) out[i] = (float)s->x[i];
}
void or_get_velocities(const or_solver* s, float* out) {
    for (int64_t i = 0; i < s->n * 3; i++) out[i] = (float)s->v[i];
}
void or_get_state64(const or_solver* s, double* x, double* v) {
    for (int64_t i = 0; i < s->n * 3; i++) {
        x[i] = (double)s->x[i];
        v[i] = (double)s->v[i];
    }
}
int64_t or_contact_count(const or_solver* s) { return s->ccount_raw < s->cmax ? s->ccount_raw : s->cmax; }
int64_t or_contact_count_raw(const or_solver* s) { return s->ccount_raw; }
void or_get_contacts(const or_solver* s, int32_t* part, int32_t* shape, float* bpos, float* bvel, float* nrm) {
    int64_t m = or_contact_count(s);
    for (int64_t t = 0; t < m; t++) {
        if (part) part[t] = s->cpart[t];
        if (shape) shape[t] = s->cshape[t];
        for (int a = 0; a < 3; a++) {
            if (bpos) bpos[t * 3 + a] = (float)s->cbpos[t * 3 + a];
            if (bvel) bvel[t * 3 + a] = (float)s->cbvel[t * 3 + a];
            if (nrm) nrm[t * 3 + a] = (float)s->cnorm[t * 3 + a];
        }
    }
}
void or_get_sorted(const or_solver* s, uint32_t* cells, uint32_t* ids) {
    if (cells) memcpy(cells, s->scells, sizeof(uint32_t) * (size_t)s->n);
    if (ids) memcpy(ids, s->sids, sizeof(uint32_t) * (size_t)s->n);
}
void or_get_cell_starts(const or_solver* s, int32_t* out) { memcpy(out, s->cstart, sizeof(int32_t) * NUM_CELLS); }
void or_get_cell_ends(const or_solver* s, int32_t* out) { memcpy(out, s->cend, sizeof(int32_t) * NUM_CELLS); }
void or_get_deltas(const or_solver* s, float* out) {
    for (int64_t i = 0; i < s->n * 3; i++) out[i] = (float)s->delta[i];
}
int64_t or_mesh_bvh_node_count(const or_solver* s, int64_t mi) {
    return (mi < 0 || mi >= s->nmesh) ? 0 : s->meshes[mi].n_nodes;
}
void or_get_mesh_bvh(const or_solver* s, int64_t mi, float* lowers, float* uppers) {
    const or_mesh* m = &s->meshes[mi];
    memcpy(lowers, m->lowers, sizeof(float) * 4 * (size_t)m->n_nodes);
    memcpy(uppers, m->uppers, sizeof(float) * 4 * (size_t)m->n_nodes);
}
int or_mesh_is_watertight_flag(const or_solver* s, int64_t mi) { return s->meshes[mi].watertight; }
float or_mesh_avg_edge(const or_solver* s, int64_t mi) { return s->meshes[mi].avg_edge; }
