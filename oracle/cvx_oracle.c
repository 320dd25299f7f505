/*
 * cvx_oracle.c -- CPU restatement of the reference's voxelization path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file is the checker for the CUDA engine in cuda_voxelizer_gb300/.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it, and only to check or to
 * time the reference algorithm on the host; the product never calls it.
 *
 * It restates, statement for statement, the reference's two CPU voxelizers
 *   cpu_voxelize_mesh        src/cpu_voxelizer.cpp:35-183  (surface, Schwarz-Seidel overlap test)
 *   cpu_voxelize_mesh_solid  src/cpu_voxelizer.cpp:241-314 (solid, parity flips along +x)
 * which are themselves restatements of the GPU kernels voxelize_triangle (src/voxelize.cu:58-190)
 * and voxelize_triangle_solid (src/voxelize_solid.cu:73-145).  The input is the flat triangle soup
 * the GPU path receives (9 floats per triangle, src/main.cpp:61-80) instead of a Trimesh.
 *
 * Arithmetic modes.  With mode == NULL the oracle reproduces the reference CPU build exactly:
 * every a*b+c is a separate rounded multiply and add (this file must be compiled with
 * -ffp-contract=off, which the build recipe passes; on aarch64 gcc would otherwise fuse them),
 * 1/|n| is 1.0f/sqrtf (helper_math.h:78-81), the linear index uses gridsize.y as row stride
 * (src/cpu_voxelizer.cpp:168,304), and the solid path uses float (y+0.5f) / (q-0.5f)
 * (src/cpu_voxelizer.cpp:285-292).  A non-NULL mode selects the GPU kernels' semantics instead:
 * an explicit fused-multiply-add pattern for each expression (the way nvcc contracts the
 * reference's helper_math expressions), the reference GPU kernel's double-promoted solid
 * arithmetic (src/voxelize_solid.cu:112-119), its index formula (src/voxelize.cu:175-178), and,
 * if mode->inv_len is given, per-triangle 1/|n| values taken from the device's own rsqrtf.
 * That mode exists so the oracle can be pinned against the reference GPU kernels too.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define FLOAT_ERROR 0.000001 /* src/voxelize_solid.cu:13, src/cpu_voxelizer.cpp:2 (a double) */

/* Byte-compatible with the reference voxinfo (src/util.h:50-69) on LP64 targets. */
typedef struct {
    float bmin[3];
    float bmax[3];
    uint32_t grid[3];
    uint32_t pad0;
    uint64_t n_tri;
    float unit[3];
    uint32_t pad1;
} ovx_info;

/* Fused-multiply-add pattern of each reference expression.  0 = no fusion (two roundings per
 * product, the CPU build); other values name which product nvcc folds into an fma. */
typedef struct {
    int cross;      /* a.y*b.z - a.z*b.y (helper_math cross): 1 = fma(a.y,b.z,-(a.z*b.y)), 2 = fma(-a.z,b.y,a.y*b.z) */
    int dot3;       /* setup dot(float3): 1 = fma(z,z',fma(x,x',y*y')), 2 = fma(z,z',fma(y,y',x*x')) */
    int dot2;       /* setup dot(float2): 1 = fma(x,x',y*y'), 2 = fma(y,y',x*x') */
    int plane;      /* per-voxel dot(n,p): 1 = fma(nz,pz,fma(nx,px,ny*py)), 2 = fma(nx,px,ny*py)+nz*pz, 3 = fma(nz,pz,fma(ny,py,nx*px)) */
    int edge_xy;    /* per-voxel dot(n_xy,p_xy): 1 = fma(a.x,px,a.y*py), 2 = fma(a.y,py,a.x*px) */
    int edge_yz;    /* per-voxel dot(n_yz,p_yz): 1 = fma(a.x,py,a.y*pz), 2 = fma(a.y,pz,a.x*py) */
    int edge_zx;    /* per-voxel dot(n_zx,p_zx): 1 = fma(a.x,pz,a.y*px), 2 = fma(a.y,px,a.x*pz) */
    int ccw;        /* solid checkCCW e0.x*e1.y - e1.x*e0.y: as cross */
    int pt;         /* solid check_point_triangle t1..t3 a*b-c*d: as cross */
    int getx;       /* solid get_x_coordinate n.y*A+n.z*B: 1 = fma(n.y,A,n.z*B), 2 = fma(n.z,B,n.y*A)
                     * (the reference GPU kernel's linear-order code uses 1, its Morton-order code 2) */
    int clip;       /* solid: keep the writes inside the grid the way the CUDA engine does where the
                     * reference writes outside its table (columns outside the grid are dropped;
                     * Morton order stops a run at x = gx; linear order continues a run into the
                     * following rows up to the last voxel of the grid) */
    const float* inv_len; /* optional per-triangle rsqrtf(dot(c,c)) values from the device */
} ovx_mode;

/* ---- small helpers --------------------------------------------------------------------- */

typedef struct { float x, y, z; } f3;
typedef struct { float x, y; } f2;

static inline f3 mk3(float x, float y, float z) { f3 r = {x, y, z}; return r; }
static inline f2 mk2(float x, float y) { f2 r = {x, y}; return r; }
static inline f3 sub3(f3 a, f3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline f2 sub2(f2 a, f2 b) { return mk2(a.x - b.x, a.y - b.y); }
/* helper_math.h:57-65 host fminf/fmaxf (ternaries) */
static inline float hfmin(float a, float b) { return a < b ? a : b; }
static inline float hfmax(float a, float b) { return a > b ? a : b; }
/* std::max<float>(0.0f, v) as called from src/cpu_voxelizer.cpp:99-125 */
static inline float smax0(float v) { return (0.0f < v) ? v : 0.0f; }

/* a*b - c*d under a fusion pattern (0: CPU, 1: first product fused, 2: second product fused) */
static inline float mul_sub(int pat, float a, float b, float c, float d) {
    if (pat == 1) return fmaf(a, b, -(c * d));
    if (pat == 2) return fmaf(-c, d, a * b);
    return a * b - c * d;
}
/* a*b + c*d */
static inline float mul_add(int pat, float a, float b, float c, float d) {
    if (pat == 1) return fmaf(a, b, c * d);
    if (pat == 2) return fmaf(c, d, a * b);
    return a * b + c * d;
}
/* helper_math dot(float3) = a.x*b.x + a.y*b.y + a.z*b.z, parsed left to right */
static inline float dot3p(int pat, f3 a, f3 b) {
    if (pat == 1) return fmaf(a.z, b.z, fmaf(a.x, b.x, a.y * b.y));
    if (pat == 2) return fmaf(a.z, b.z, fmaf(a.y, b.y, a.x * b.x));
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
static inline float plane_dot(int pat, f3 n, f3 p) {
    if (pat == 1) return fmaf(n.z, p.z, fmaf(n.x, p.x, n.y * p.y));
    if (pat == 2) return fmaf(n.x, p.x, n.y * p.y) + n.z * p.z;
    if (pat == 3) return fmaf(n.z, p.z, fmaf(n.y, p.y, n.x * p.x));
    return n.x * p.x + n.y * p.y + n.z * p.z;
}

/* static_cast<int>(float): x86 cvttss2si gives INT_MIN out of range (CPU build); the GPU's
 * cvt.rzi.s32.f32 saturates and maps NaN to 0. Only reachable for coordinates far outside the
 * grid. */
static inline int f2i(float v, int gpu) {
    if (gpu) {
        if (v != v) return 0;
        if (v >= 2147483648.0f) return 2147483647;
        if (v <= -2147483648.0f) return (-2147483647 - 1);
        return (int)v;
    }
    if (!(v > -2147483904.0f && v < 2147483648.0f)) return (-2147483647 - 1);
    return (int)v;
}
/* int(double) with the device's saturating conversion (cvt.rzi.s32.f64); NaN gives 0. */
static inline int d2i(double v) {
    if (v != v) return 0;
    if (v >= 2147483647.0) return 2147483647;
    if (v <= -2147483648.0) return (-2147483647 - 1);
    return (int)v;
}
static inline int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); } /* helper_math clamp: max(a, min(f, b)) */

/* ---- Morton LUT encode (src/voxelize.cuh:20-34, src/cpu_voxelizer.cpp:18-32) -------------- */

static uint32_t lut_x[256], lut_y[256], lut_z[256];
static int lut_ready = 0;

/* The tables of src/morton_LUTs.h are the 3-way bit spread of the byte: bit i of the index goes
 * to bit 3i (x), 3i+1 (y) and 3i+2 (z).  tests/ checks this against the reference's tables. */
static void init_luts(void) {
    if (lut_ready) return;
    for (uint32_t v = 0; v < 256; v++) {
        uint32_t s = 0;
        for (int i = 0; i < 8; i++) s |= ((v >> i) & 1u) << (3 * i);
        lut_x[v] = s; lut_y[v] = s << 1; lut_z[v] = s << 2;
    }
    lut_ready = 1;
}

uint64_t ovx_morton_encode(uint32_t x, uint32_t y, uint32_t z) {
    init_luts();
    uint64_t answer = 0;
    answer = (uint64_t)(lut_z[(z >> 16) & 0xFF] | lut_y[(y >> 16) & 0xFF] | lut_x[(x >> 16) & 0xFF]);
    answer = answer << 48 | lut_z[(z >> 8) & 0xFF] | lut_y[(y >> 8) & 0xFF] | lut_x[(x >> 8) & 0xFF];
    answer = answer << 24 | lut_z[z & 0xFF] | lut_y[y & 0xFF] | lut_x[x & 0xFF];
    return answer;
}

void ovx_morton_lut(int axis, uint32_t out[256]) {
    init_luts();
    memcpy(out, axis == 0 ? lut_x : (axis == 1 ? lut_y : lut_z), sizeof(lut_x));
}

/* ---- bit writes (src/cpu_voxelizer.cpp:7-15, :186-194) ------------------------------------ */

static int g_parallel = 0;

/* Counting pass (ovx_count_atomics, serial only): surface bit writes record their word instead of
 * writing it; solid column hits are counted before their bits are written. */
static int g_count = 0;
static uint64_t* g_words = NULL;
static size_t g_nwords = 0, g_capwords = 0;
static uint64_t g_hits = 0;

static void count_word(uint64_t w) {
    if (g_nwords == g_capwords) {
        size_t cap = g_capwords ? 2 * g_capwords : 4096;
        uint64_t* p = (uint64_t*)realloc(g_words, cap * sizeof(uint64_t));
        if (!p) abort();
        g_words = p;
        g_capwords = cap;
    }
    g_words[g_nwords++] = w;
}

static inline void set_bit(uint32_t* table, uint64_t index) {
    uint64_t w = index / 32u;
    uint32_t mask = 1u << (31u - (uint32_t)(index % 32u));
    if (g_count) {
        count_word(w);
        return;
    }
    if (g_parallel) {
#ifdef _OPENMP
#pragma omp critical
#endif
        { table[w] = table[w] | mask; }
    } else {
        table[w] |= mask;
    }
}
static inline void set_bit_xor(uint32_t* table, uint64_t index) {
    uint64_t w = index / 32u;
    uint32_t mask = 1u << (31u - (uint32_t)(index % 32u));
    if (g_parallel) {
#ifdef _OPENMP
#pragma omp critical
#endif
        { table[w] = table[w] ^ mask; }
    } else {
        table[w] ^= mask;
    }
}

/* ---- surface: one triangle (src/cpu_voxelizer.cpp:54-175; src/voxelize.cu:66-188) ---------- */

static void surface_triangle(const ovx_info* info, const float* tri, uint64_t t, uint32_t* table,
                             int morton, const ovx_mode* m) {
    const int gpu = m != NULL;
    const int pc = gpu ? m->cross : 0, p3 = gpu ? m->dot3 : 0, p2 = gpu ? m->dot2 : 0;
    const f3 unit = mk3(info->unit[0], info->unit[1], info->unit[2]);
    const f3 delta_p = unit;
    f3 c = mk3(0.0f, 0.0f, 0.0f);
    const int gmx = (int)info->grid[0] - 1, gmy = (int)info->grid[1] - 1, gmz = (int)info->grid[2] - 1;
    const f3 bmin = mk3(info->bmin[0], info->bmin[1], info->bmin[2]);

    /* vertices moved to the bbox origin (src/cpu_voxelizer.cpp:40-45 / src/voxelize.cu:71-73) */
    f3 v0 = sub3(mk3(tri[0], tri[1], tri[2]), bmin);
    f3 v1 = sub3(mk3(tri[3], tri[4], tri[5]), bmin);
    f3 v2 = sub3(mk3(tri[6], tri[7], tri[8]), bmin);
    f3 e0 = sub3(v1, v0), e1 = sub3(v2, v1), e2 = sub3(v0, v2);
    /* n = normalize(cross(e0, e1)) (helper_math.h:1325-1329, :1436-1439) */
    f3 cr = mk3(mul_sub(pc, e0.y, e1.z, e0.z, e1.y), mul_sub(pc, e0.z, e1.x, e0.x, e1.z),
                mul_sub(pc, e0.x, e1.y, e0.y, e1.x));
    float inv = (gpu && m->inv_len) ? m->inv_len[t] : 1.0f / sqrtf(dot3p(p3, cr, cr));
    f3 n = mk3(cr.x * inv, cr.y * inv, cr.z * inv);

    /* triangle bbox in grid coordinates (src/cpu_voxelizer.cpp:76-80) */
    f3 wmin = mk3(hfmin(v0.x, hfmin(v1.x, v2.x)), hfmin(v0.y, hfmin(v1.y, v2.y)), hfmin(v0.z, hfmin(v1.z, v2.z)));
    f3 wmax = mk3(hfmax(v0.x, hfmax(v1.x, v2.x)), hfmax(v0.y, hfmax(v1.y, v2.y)), hfmax(v0.z, hfmax(v1.z, v2.z)));
    if (gpu) { /* device fminf/fmaxf return the non-NaN operand */
        wmin = mk3(fminf(v0.x, fminf(v1.x, v2.x)), fminf(v0.y, fminf(v1.y, v2.y)), fminf(v0.z, fminf(v1.z, v2.z)));
        wmax = mk3(fmaxf(v0.x, fmaxf(v1.x, v2.x)), fmaxf(v0.y, fmaxf(v1.y, v2.y)), fmaxf(v0.z, fmaxf(v1.z, v2.z)));
    }
    int bx0 = clampi(f2i(wmin.x / unit.x, gpu), 0, gmx), by0 = clampi(f2i(wmin.y / unit.y, gpu), 0, gmy), bz0 = clampi(f2i(wmin.z / unit.z, gpu), 0, gmz);
    int bx1 = clampi(f2i(wmax.x / unit.x, gpu), 0, gmx), by1 = clampi(f2i(wmax.y / unit.y, gpu), 0, gmy), bz1 = clampi(f2i(wmax.z / unit.z, gpu), 0, gmz);

    /* plane test properties (src/cpu_voxelizer.cpp:83-87) */
    if (n.x > 0.0f) c.x = unit.x;
    if (n.y > 0.0f) c.y = unit.y;
    if (n.z > 0.0f) c.z = unit.z;
    float d1 = dot3p(p3, n, sub3(c, v0));
    float d2 = dot3p(p3, n, sub3(sub3(delta_p, c), v0));

    /* projection test properties (src/cpu_voxelizer.cpp:91-125) */
    f2 nxy[3] = {mk2(-1.0f * e0.y, e0.x), mk2(-1.0f * e1.y, e1.x), mk2(-1.0f * e2.y, e2.x)};
    if (n.z < 0.0f) for (int i = 0; i < 3; i++) nxy[i] = mk2(-nxy[i].x, -nxy[i].y);
    f2 nyz[3] = {mk2(-1.0f * e0.z, e0.y), mk2(-1.0f * e1.z, e1.y), mk2(-1.0f * e2.z, e2.y)};
    if (n.x < 0.0f) for (int i = 0; i < 3; i++) nyz[i] = mk2(-nyz[i].x, -nyz[i].y);
    f2 nzx[3] = {mk2(-1.0f * e0.x, e0.z), mk2(-1.0f * e1.x, e1.z), mk2(-1.0f * e2.x, e2.z)};
    if (n.y < 0.0f) for (int i = 0; i < 3; i++) nzx[i] = mk2(-nzx[i].x, -nzx[i].y);
    const f3 vv[3] = {v0, v1, v2};
    float dxy[3], dyz[3], dzx[3];
    for (int i = 0; i < 3; i++) {
        dxy[i] = (-1.0f * mul_add(p2, nxy[i].x, vv[i].x, nxy[i].y, vv[i].y)) + smax0(unit.x * nxy[i].x) + smax0(unit.y * nxy[i].y);
        dyz[i] = (-1.0f * mul_add(p2, nyz[i].x, vv[i].y, nyz[i].y, vv[i].z)) + smax0(unit.y * nyz[i].x) + smax0(unit.z * nyz[i].y);
        dzx[i] = (-1.0f * mul_add(p2, nzx[i].x, vv[i].z, nzx[i].y, vv[i].x)) + smax0(unit.x * nzx[i].x) + smax0(unit.z * nzx[i].y);
    }
    const int pp = gpu ? m->plane : 0, pxy = gpu ? m->edge_xy : 0, pyz = gpu ? m->edge_yz : 0, pzx = gpu ? m->edge_zx : 0;

    /* voxel loop (src/cpu_voxelizer.cpp:128-175) */
    for (int z = bz0; z <= bz1; z++) {
        for (int y = by0; y <= by1; y++) {
            for (int x = bx0; x <= bx1; x++) {
                f3 p = mk3((float)x * unit.x, (float)y * unit.y, (float)z * unit.z);
                float nDOTp = plane_dot(pp, n, p);
                if (((nDOTp + d1) * (nDOTp + d2)) > 0.0f) continue;
                int fail = 0;
                for (int i = 0; i < 3 && !fail; i++) if ((mul_add(pxy, nxy[i].x, p.x, nxy[i].y, p.y) + dxy[i]) < 0.0f) fail = 1;
                for (int i = 0; i < 3 && !fail; i++) if ((mul_add(pyz, nyz[i].x, p.y, nyz[i].y, p.z) + dyz[i]) < 0.0f) fail = 1;
                for (int i = 0; i < 3 && !fail; i++) if ((mul_add(pzx, nzx[i].x, p.z, nzx[i].y, p.x) + dzx[i]) < 0.0f) fail = 1;
                if (fail) continue;
                uint64_t loc;
                if (morton) {
                    loc = ovx_morton_encode((uint32_t)x, (uint32_t)y, (uint32_t)z);
                } else if (gpu) { /* src/voxelize.cu:175-178 */
                    loc = (uint64_t)x + (uint64_t)y * info->grid[0] + (uint64_t)z * ((uint64_t)info->grid[1] * info->grid[0]);
                } else {          /* src/cpu_voxelizer.cpp:168 */
                    loc = (uint64_t)x + (uint64_t)y * info->grid[1] + (uint64_t)z * (uint64_t)info->grid[1] * (uint64_t)info->grid[2];
                }
                set_bit(table, loc);
            }
        }
    }
}

/* ---- solid helpers (src/cpu_voxelizer.cpp:196-238; src/voxelize_solid.cu:24-70) ----------- */

static inline int top_left_edge(f2 v0, f2 v1) { return (v1.y < v0.y) || (v1.y == v0.y && v0.x > v1.x); }

static inline int check_ccw(int pat, f2 v0, f2 v1, f2 v2) {
    f2 e0 = sub2(v1, v0), e1 = sub2(v2, v0);
    float result = mul_sub(pat, e0.x, e1.y, e1.x, e0.y);
    return result > 0;
}

static inline int check_point_triangle(int pat, f2 v0, f2 v1, f2 v2, f2 point) {
    f2 PA = sub2(point, v0), PB = sub2(point, v1), PC = sub2(point, v2);
    float t1 = mul_sub(pat, PA.x, PB.y, PA.y, PB.x);
    if (((double)fabsf(t1)) < FLOAT_ERROR && PA.x * PB.x <= 0 && PA.y * PB.y <= 0) return 1;
    float t2 = mul_sub(pat, PB.x, PC.y, PB.y, PC.x);
    if (((double)fabsf(t2)) < FLOAT_ERROR && PB.x * PC.x <= 0 && PB.y * PC.y <= 0) return 2;
    float t3 = mul_sub(pat, PC.x, PA.y, PC.y, PA.x);
    if (((double)fabsf(t3)) < FLOAT_ERROR && PC.x * PA.x <= 0 && PC.y * PA.y <= 0) return 3;
    if (t1 * t2 > 0 && t1 * t3 > 0) return 0;
    return -1;
}

static inline float get_x_coordinate(int pat, f3 n, f3 v0, f2 point) {
    return (-mul_add(pat, n.y, point.x - v0.y, n.z, point.y - v0.z) / n.x + v0.x);
}

/* ---- solid: one triangle (src/cpu_voxelizer.cpp:254-311; src/voxelize_solid.cu:78-143) ------- */

static void solid_triangle(const ovx_info* info, const float* tri, uint64_t t, uint32_t* table,
                           uint64_t table_words, int morton, const ovx_mode* m) {
    const int gpu = m != NULL;
    const int pc = gpu ? m->cross : 0, p3 = gpu ? m->dot3 : 0, pw = gpu ? m->ccw : 0, pg = gpu ? m->getx : 0;
    const int pp = gpu ? m->pt : 0, clip = gpu && m->clip;
    const uint64_t total_bits = (uint64_t)info->grid[0] * info->grid[1] * info->grid[2];
    const f3 bmin = mk3(info->bmin[0], info->bmin[1], info->bmin[2]);
    const f3 unit = mk3(info->unit[0], info->unit[1], info->unit[2]);
    f3 v0 = sub3(mk3(tri[0], tri[1], tri[2]), bmin);
    f3 v1 = sub3(mk3(tri[3], tri[4], tri[5]), bmin);
    f3 v2 = sub3(mk3(tri[6], tri[7], tri[8]), bmin);
    f3 e0 = sub3(v1, v0), e1 = sub3(v2, v1);
    f3 cr = mk3(mul_sub(pc, e0.y, e1.z, e0.z, e1.y), mul_sub(pc, e0.z, e1.x, e0.x, e1.z),
                mul_sub(pc, e0.x, e1.y, e0.y, e1.x));
    float inv = (gpu && m->inv_len) ? m->inv_len[t] : 1.0f / sqrtf(dot3p(p3, cr, cr));
    f3 n = mk3(cr.x * inv, cr.y * inv, cr.z * inv);
    if (((double)fabsf(n.x)) < FLOAT_ERROR) return;

    f2 v0_yz = mk2(v0.y, v0.z), v1_yz = mk2(v1.y, v1.z), v2_yz = mk2(v2.y, v2.z);
    if (!check_ccw(pw, v0_yz, v1_yz, v2_yz)) { f2 v3 = v1_yz; v1_yz = v2_yz; v2_yz = v3; }
    f2 bbox_max, bbox_min;
    if (gpu) {
        bbox_max = mk2(fmaxf(v0_yz.x, fmaxf(v1_yz.x, v2_yz.x)), fmaxf(v0_yz.y, fmaxf(v1_yz.y, v2_yz.y)));
        bbox_min = mk2(fminf(v0_yz.x, fminf(v1_yz.x, v2_yz.x)), fminf(v0_yz.y, fminf(v1_yz.y, v2_yz.y)));
    } else {
        bbox_max = mk2(hfmax(v0_yz.x, hfmax(v1_yz.x, v2_yz.x)), hfmax(v0_yz.y, hfmax(v1_yz.y, v2_yz.y)));
        bbox_min = mk2(hfmin(v0_yz.x, hfmin(v1_yz.x, v2_yz.x)), hfmin(v0_yz.y, hfmin(v1_yz.y, v2_yz.y)));
    }
    f2 gmax, gmin;
    if (gpu) { /* src/voxelize_solid.cu:112-113: the 0.5 literal promotes to double */
        gmax = mk2((float)floor((double)(bbox_max.x / unit.y) - 0.5), (float)floor((double)(bbox_max.y / unit.z) - 0.5));
        gmin = mk2((float)ceil((double)(bbox_min.x / unit.y) - 0.5), (float)ceil((double)(bbox_min.y / unit.z) - 0.5));
    } else {   /* src/cpu_voxelizer.cpp:285-286: float throughout */
        gmax = mk2(floorf(bbox_max.x / unit.y - 0.5f), floorf(bbox_max.y / unit.z - 0.5f));
        gmin = mk2(ceilf(bbox_min.x / unit.y - 0.5f), ceilf(bbox_min.y / unit.z - 0.5f));
    }
    /* Column loops as in the reference; bounded at 2^24 so that non-finite bounds (garbage input)
     * cannot run away. */
    for (int y = f2i(gmin.x, gpu); (float)y <= gmax.x && y < (1 << 24); y++) {
        for (int z = f2i(gmin.y, gpu); (float)z <= gmax.y && z < (1 << 24); z++) {
            f2 point;
            if (gpu) point = mk2((float)(((double)y + 0.5) * (double)unit.y), (float)(((double)z + 0.5) * (double)unit.z));
            else point = mk2(((float)y + 0.5f) * unit.y, ((float)z + 0.5f) * unit.z);
            if (clip && (y < 0 || z < 0 || (uint32_t)y >= info->grid[1] || (uint32_t)z >= info->grid[2])) continue;
            int checknum = check_point_triangle(pp, v0_yz, v1_yz, v2_yz, point);
            if ((checknum == 1 && top_left_edge(v0_yz, v1_yz)) || (checknum == 2 && top_left_edge(v1_yz, v2_yz)) ||
                (checknum == 3 && top_left_edge(v2_yz, v0_yz)) || (checknum == 0)) {
                int xmax = d2i((double)(get_x_coordinate(pg, n, v0, point) / unit.x) - 0.5);
                /* The CPU build stores xmax as unsigned (src/cpu_voxelizer.cpp:296-297); the GPU
                 * kernel keeps it signed (src/voxelize_solid.cu:123-124).  They only differ for
                 * hits left of the grid, where the CPU loop runs away; both stop here. */
                if (xmax < 0) continue;
                if (g_count) {
                    g_hits++;
                    continue;
                }
                if (clip && !morton && !g_parallel) {
                    /* the same bits as the loop below (x = 0..xmax of the row, continuing into the
                     * following rows, up to the grid's last voxel), XORed a word at a time */
                    const uint64_t lo = (uint64_t)y * info->grid[0] + (uint64_t)z * ((uint64_t)info->grid[1] * info->grid[0]);
                    if (lo >= total_bits) continue;
                    const uint64_t hi = lo + (uint64_t)xmax < total_bits ? lo + (uint64_t)xmax : total_bits - 1;
                    for (uint64_t w = lo / 32u; w <= hi / 32u; w++) {
                        const uint32_t a = w == lo / 32u ? (uint32_t)(lo % 32u) : 0u;
                        const uint32_t b = w == hi / 32u ? (uint32_t)(hi % 32u) : 31u;
                        table[w] ^= (0xFFFFFFFFu >> a) & (0xFFFFFFFFu << (31u - b));
                    }
                    continue;
                }
                for (int64_t x = 0; x <= xmax; x++) {
                    uint64_t loc;
                    if (clip && morton && (uint64_t)x >= info->grid[0]) break;
                    if (morton) {
                        loc = ovx_morton_encode((uint32_t)x, (uint32_t)y, (uint32_t)z);
                    } else if (gpu) {
                        loc = (uint64_t)x + (uint64_t)(int64_t)y * info->grid[0] + (uint64_t)(int64_t)z * ((uint64_t)info->grid[1] * info->grid[0]);
                    } else {
                        loc = (uint64_t)x + (uint64_t)(int64_t)y * info->grid[1] + (uint64_t)(int64_t)z * (uint64_t)info->grid[1] * (uint64_t)info->grid[2];
                    }
                    if (clip && loc >= total_bits) break;
                    if (loc / 32u >= table_words) continue; /* the reference writes out of bounds here */
                    set_bit_xor(table, loc);
                }
            }
        }
    }
}

/* ---- public entry points -------------------------------------------------------------------- */

static uint64_t words_for(const ovx_info* info) {
    uint64_t bits = (uint64_t)info->grid[0] * info->grid[1] * info->grid[2];
    return (bits + 31u) / 32u;
}

/* Serial restatement: surface (src/cpu_voxelizer.cpp:35) or solid (:241). */
void ovx_voxelize(const ovx_info* info, const float* tris, uint32_t* table, int morton, int solid, const ovx_mode* mode) {
    init_luts();
    g_parallel = 0;
    uint64_t words = words_for(info);
    for (uint64_t t = 0; t < info->n_tri; t++) {
        if (solid) solid_triangle(info, tris + 9 * t, t, table, words, morton, mode);
        else surface_triangle(info, tris + 9 * t, t, table, morton, mode);
    }
}

/* dot(c, c) of each triangle's cross product c = cross(e0, e1) under mode m's patterns (the value
 * the reference kernels pass to rsqrtf in normalize, helper_math.h:1436-1439), so that a caller can
 * evaluate the device's rsqrtf on it and hand the results back as m->inv_len. */
void ovx_len2(const ovx_info* info, const float* tris, const ovx_mode* m, float* out) {
    const int pc = m ? m->cross : 0, p3 = m ? m->dot3 : 0;
    const f3 bmin = mk3(info->bmin[0], info->bmin[1], info->bmin[2]);
    for (uint64_t t = 0; t < info->n_tri; t++) {
        const float* tri = tris + 9 * t;
        f3 v0 = sub3(mk3(tri[0], tri[1], tri[2]), bmin);
        f3 v1 = sub3(mk3(tri[3], tri[4], tri[5]), bmin);
        f3 v2 = sub3(mk3(tri[6], tri[7], tri[8]), bmin);
        f3 e0 = sub3(v1, v0), e1 = sub3(v2, v1);
        f3 cr = mk3(mul_sub(pc, e0.y, e1.z, e0.z, e1.y), mul_sub(pc, e0.z, e1.x, e0.x, e1.z),
                    mul_sub(pc, e0.x, e1.y, e0.y, e1.x));
        out[t] = dot3p(p3, cr, cr);
    }
}

static int cmp_u64(const void* a, const void* b) {
    uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y);
}

/* The atomic term of the roofline, counted exactly from the mesh: surface, the number of distinct
 * table words each triangle sets a bit in, summed over triangles; solid, the number of column hits
 * (every hit flips a run of bits in one row).  Serial; the table is not written. */
uint64_t ovx_count_atomics(const ovx_info* info, const float* tris, int morton, int solid) {
    init_luts();
    g_parallel = 0;
    g_count = 1;
    g_hits = 0;
    uint64_t total = 0, words = words_for(info);
    for (uint64_t t = 0; t < info->n_tri; t++) {
        if (solid) {
            solid_triangle(info, tris + 9 * t, t, NULL, words, morton, NULL);
            continue;
        }
        g_nwords = 0;
        surface_triangle(info, tris + 9 * t, t, NULL, morton, NULL);
        if (g_nwords > 1) qsort(g_words, g_nwords, sizeof(uint64_t), cmp_u64);
        for (size_t i = 0; i < g_nwords; i++)
            if (i == 0 || g_words[i] != g_words[i - 1]) total++;
    }
    if (solid) total = g_hits;
    g_count = 0;
    free(g_words);
    g_words = NULL;
    g_nwords = g_capwords = 0;
    return total;
}

/* The same restatement run the way the reference runs it on the host: an OpenMP parallel for
 * over triangles with every bit write inside `omp critical` (src/cpu_voxelizer.cpp:11-14, :53,
 * :190-193, :253).  This is the "port" CPU baseline used when the reference's own build cannot
 * run on the host (it is compiled for another architecture). */
void ovx_voxelize_omp(const ovx_info* info, const float* tris, uint32_t* table, int morton, int solid, int threads) {
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    init_luts();
    g_parallel = 1;
    uint64_t words = words_for(info);
    int64_t n = (int64_t)info->n_tri;
#ifdef _OPENMP
#pragma omp parallel for
#endif
    for (int64_t t = 0; t < n; t++) {
        if (solid) solid_triangle(info, tris + 9 * t, (uint64_t)t, table, words, morton, NULL);
        else surface_triangle(info, tris + 9 * t, (uint64_t)t, table, morton, NULL);
    }
    g_parallel = 0;
}

int ovx_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ---- output writers (src/util_io.cpp) ------------------------------------------------------ */

/* checkVoxel (src/util.h:25-38): linear index x + y*gx + z*gx*gy, bit 31 - index%32. */
static int check_voxel(const uint32_t* t, const ovx_info* info, uint64_t x, uint64_t y, uint64_t z) {
    uint64_t loc = x + y * info->grid[0] + z * (uint64_t)info->grid[0] * info->grid[1];
    return (t[loc / 32u] >> (31u - (uint32_t)(loc % 32u))) & 1u;
}

/* write_binvox's data section (src/util_io.cpp:219-245): x, then z, then y; the first voxel's
 * value, then a count each time the value changes or the count reaches 255, then the value, and
 * the last count.  Writes at most `cap` bytes to out; returns the number of bytes produced. */
uint64_t ovx_binvox_payload(const ovx_info* info, const uint32_t* table, uint8_t* out, uint64_t cap) {
    uint64_t n = 0;
#define OVX_PUT(b) do { if (n < cap) out[n] = (uint8_t)(b); n++; } while (0)
    uint8_t current = 0, seen = 0;
    for (uint64_t x = 0; x < info->grid[0]; x++) {
        for (uint64_t z = 0; z < info->grid[2]; z++) {
            for (uint64_t y = 0; y < info->grid[1]; y++) {
                if (x == 0 && y == 0 && z == 0) {
                    current = (uint8_t)check_voxel(table, info, 0, 0, 0);
                    OVX_PUT(current);
                    seen = 1;
                    continue;
                }
                uint8_t next = (uint8_t)check_voxel(table, info, x, y, z);
                if (next != current || seen == 255) {
                    OVX_PUT(seen);
                    seen = 1;
                    current = next;
                    OVX_PUT(current);
                } else {
                    seen++;
                }
            }
        }
    }
    OVX_PUT(seen);
#undef OVX_PUT
    return n;
}

/* write_vox's voxel loop (src/util_io.cpp:264-280): x, then y over [0, gz), then z over [0, gy);
 * every set voxel becomes AddVoxel(x, -z + gz, y).  Writes at most cap triples; returns the count. */
uint64_t ovx_vox_list(const ovx_info* info, const uint32_t* table, int32_t* out, uint64_t cap) {
    uint64_t n = 0;
    for (uint64_t x = 0; x < info->grid[0]; x++) {
        for (uint64_t y = 0; y < info->grid[2]; y++) {
            for (uint64_t z = 0; z < info->grid[1]; z++) {
                if (check_voxel(table, info, x, y, z)) {
                    if (n < cap) {
                        out[3 * n] = (int32_t)x;
                        out[3 * n + 1] = (int32_t)(-(int64_t)z + (int64_t)info->grid[2]);
                        out[3 * n + 2] = (int32_t)y;
                    }
                    n++;
                }
            }
        }
    }
    return n;
}

/* createMeshBBCube (src/util.h:80-110) on float3 bounds. */
void ovx_mesh_bbcube(const float in_min[3], const float in_max[3], float out_min[3], float out_max[3]) {
    float len[3] = {in_max[0] - in_min[0], in_max[1] - in_min[1], in_max[2] - in_min[2]};
    /* std::max(lengths.x, std::max(lengths.y, lengths.z)) with std::max(a,b) = (a < b) ? b : a */
    float myz = (len[1] < len[2]) ? len[2] : len[1];
    float mx = (len[0] < myz) ? myz : len[0];
    for (int i = 0; i < 3; i++) { out_min[i] = in_min[i]; out_max[i] = in_max[i]; }
    for (int i = 0; i < 3; i++) {
        if (mx != len[i]) {
            float delta = mx - len[i];
            out_min[i] = in_min[i] - (delta / 2.0f);
            out_max[i] = in_max[i] + (delta / 2.0f);
        }
    }
    float eps[3];
    for (int i = 0; i < 3; i++) eps[i] = (out_max[i] - out_min[i]) / 10001.0f;
    for (int i = 0; i < 3; i++) { out_min[i] -= eps[i]; out_max[i] += eps[i]; }
}

/* voxinfo constructor (src/util.h:56-61). */
void ovx_info_init(ovx_info* info, const float bmin[3], const float bmax[3], const uint32_t grid[3], uint64_t n_tri) {
    memset(info, 0, sizeof(*info));
    for (int i = 0; i < 3; i++) {
        info->bmin[i] = bmin[i]; info->bmax[i] = bmax[i]; info->grid[i] = grid[i];
        info->unit[i] = (bmax[i] - bmin[i]) / (float)grid[i];
    }
    info->n_tri = n_tri;
}
