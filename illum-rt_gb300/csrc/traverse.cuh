// Device-side traversal of the flattened BVH (layout in bvh_builder.hpp).
//
// Results are bit-identical to the reference CPU tracer (rt/cpu/bvh2.cpp:71-189) on the same
// BVH and rays:
//   * the slab test follows intersect4 (libgi/intersect.h:230-267) with the ray's [t_min, t_max]
//     range and the same compare-and-select structure (so NaN cases come out the same);
//   * the triangle test is the reference's Cramer/Shirley test (libgi/intersect.h:19-74) with
//     every product, sum and quotient rounded exactly as written (__fmul_rn, __fadd_rn,
//     __fdiv_rn; nothing is contracted into an FMA);
//   * children are visited in the reference's order (near child first, ties to the right),
//     boxes are culled against the closest hit when they are tested (not when popped), and a
//     hit replaces the closest one only if strictly nearer, so the first of two equal hits wins.
#pragma once
#include <cfloat>
#include <cstdint>

#include "grt_internal.hpp"

namespace grt {

// A ray: origin and 1/d (libgi/rt.h:24-31) in packed f32x2 pairs, the operands of the slab
// test (low word first): (o.x, o.y), (o.z, o.z), (1/d.x, 1/d.y), (1/d.z, 1/d.z).
struct ray_t {
    uint64_t oxy, ozz, ixy, izz;
    float dx, dy, dz, tmin, tmax;
    __device__ __forceinline__ float ox() const;
    __device__ __forceinline__ float oy() const;
    __device__ __forceinline__ float oz() const;
    __device__ __forceinline__ float ix() const;
    __device__ __forceinline__ float iy() const;
    __device__ __forceinline__ float iz() const;
};

// Two f32 values in one 64-bit register, `lo` in the low word (the lower address in memory).
__device__ __forceinline__ uint64_t pk2(float lo, float hi) {
    uint64_t v;
    asm("mov.b64 %0, {%1, %2};" : "=l"(v) : "f"(lo), "f"(hi));
    return v;
}
__device__ __forceinline__ void upk2(uint64_t v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
// Packed subtraction and product (sm_100 and later): each of the two lanes is rounded to
// nearest as the scalar sub.rn.f32 / mul.rn.f32 would round it, so results keep their bits.
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// Three-input minimum and maximum (sm_100 and later), used on operands that are never NaN.
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

__device__ __forceinline__ float lo2(uint64_t v) {
    float a, b;
    upk2(v, a, b);
    return a;
}
__device__ __forceinline__ float hi2(uint64_t v) {
    float a, b;
    upk2(v, a, b);
    return b;
}
__device__ __forceinline__ float ray_t::ox() const { return lo2(oxy); }
__device__ __forceinline__ float ray_t::oy() const { return hi2(oxy); }
__device__ __forceinline__ float ray_t::oz() const { return lo2(ozz); }
__device__ __forceinline__ float ray_t::ix() const { return lo2(ixy); }
__device__ __forceinline__ float ray_t::iy() const { return hi2(ixy); }
__device__ __forceinline__ float ray_t::iz() const { return lo2(izz); }

// A ray from its origin, direction and [t_min, t_max]; ray::ray computes id = 1/d in IEEE
// float (libgi/rt.h:28).
__device__ __forceinline__ ray_t make_ray(float ox, float oy, float oz, float dx, float dy, float dz, float tmin,
                                          float tmax) {
    ray_t r;
    const float ix = __fdiv_rn(1.0f, dx), iy = __fdiv_rn(1.0f, dy), iz = __fdiv_rn(1.0f, dz);
    r.oxy = pk2(ox, oy);
    r.ozz = pk2(oz, oz);
    r.ixy = pk2(ix, iy);
    r.izz = pk2(iz, iz);
    r.dx = dx;
    r.dy = dy;
    r.dz = dz;
    r.tmin = tmin;
    r.tmax = tmax;
    return r;
}

// The largest float below x (x not NaN): t < x exactly when t <= below(x), for any t that is
// not NaN.
__device__ __forceinline__ float below(float x) {
    const uint32_t u = __float_as_uint(x);
    return __uint_as_float(x > 0.f ? u - 1u : (x == 0.f ? 0x80000001u : u + 1u));
}

struct hit_t {
    float t, b, g;
    uint32_t ref;
    uint32_t rec;  // triangle record of the hit (device layout index)
};

__device__ __forceinline__ ray_t load_ray(const float4 *__restrict__ rays, uint32_t i) {
    const float4 a = __ldg(rays + 2 * (size_t)i), d = __ldg(rays + 2 * (size_t)i + 1);
    return make_ray(a.x, a.y, a.z, d.x, d.y, d.z, a.w, d.w);
}

__device__ __forceinline__ bool finite_nonzero(float x) { return isfinite(x) && x != 0.f; }

// A ray is "plain" when no slab product (box - o) * (1/d) can be NaN: o finite and every
// 1/d finite and non-zero. Then min/max instructions give exactly the reference's selects
// (they differ only on NaN operands, and on the sign of zero, which no comparison sees), and
// the traversal takes slab2 instead of slab.
__device__ __forceinline__ bool ray_is_plain(const ray_t &r) {
    return finite_nonzero(r.ix()) && finite_nonzero(r.iy()) && finite_nonzero(r.iz()) && isfinite(r.ox()) &&
           isfinite(r.oy()) && isfinite(r.oz());
}

// The reference's slab test, intersect4 (libgi/intersect.h:230-267), with glm's min / max as the
// selects (y < x) ? y : x and (x < y) ? y : x, for rays that are not plain.
__device__ __forceinline__ bool slab(float lx, float ly, float lz, float hx, float hy, float hz, const ray_t &r,
                                     float &tnear) {
    const float ax = __fmul_rn(__fsub_rn(lx, r.ox()), r.ix()), bx = __fmul_rn(__fsub_rn(hx, r.ox()), r.ix());
    const float ay = __fmul_rn(__fsub_rn(ly, r.oy()), r.iy()), by = __fmul_rn(__fsub_rn(hy, r.oy()), r.iy());
    const float az = __fmul_rn(__fsub_rn(lz, r.oz()), r.iz()), bz = __fmul_rn(__fsub_rn(hz, r.oz()), r.iz());
    const float t1x = (ax < bx) ? ax : bx, t2x = (bx < ax) ? ax : bx;
    const float t1y = (ay < by) ? ay : by, t2y = (by < ay) ? ay : by;
    const float t1z = (az < bz) ? az : bz, t2z = (bz < az) ? az : bz;
    float t1 = (t1x < t1y) ? t1y : t1x;
    t1 = (t1z < t1) ? t1 : t1z;
    float t2 = (t2x < t2y) ? t2x : t2y;
    t2 = (t2z < t2) ? t2z : t2;
    tnear = t1;
    return !(t1 > t2) && !(t2 < r.tmin) && !(t1 > r.tmax);
}

// The slab test of a plain ray (ray_is_plain) against one child record of a binary node,
// (lo.x, lo.y, hi.x, hi.y) in `xy` pairs and (lo.z, hi.z) in `z`: the six differences and six
// products of slab() as three packed operations each, the same bits. With no NaN among the
// products, slab()'s !(t1 > t2) && !(t1 > t_max), and the closest-hit cull t1 < t_closest, are
// together t1 <= min(t2, lim) for lim = t_max (any hit) or min(t_max, below(t_closest)), a
// NaN t_max dropping out of the minimum as it drops out of slab()'s comparison.
__device__ __forceinline__ bool slab2(uint64_t xy_lo, uint64_t xy_hi, uint64_t z, const ray_t &r, float lim,
                                      float &tnear) {
    float ax, ay, bx, by, az, bz;
    upk2(mul2(sub2(xy_lo, r.oxy), r.ixy), ax, ay);
    upk2(mul2(sub2(xy_hi, r.oxy), r.ixy), bx, by);
    upk2(mul2(sub2(z, r.ozz), r.izz), az, bz);
    const float t1 = max3f(fminf(ax, bx), fminf(ay, by), fminf(az, bz));
    const float t2 = min3f(fmaxf(ax, bx), fmaxf(ay, by), fmaxf(az, bz));
    tnear = t1;
    return t1 <= fminf(t2, lim) && !(t2 < r.tmin);
}

// Cramer's rule test of the reference (libgi/intersect.h:36-67) on a triangle record
// (v0, v0 - v1, v0 - v2), every operation rounded as the reference rounds it.
//
// Before the three IEEE divisions, cheap tests discard cases whose rounded quotients could not
// pass the reference's conditions anyway, so the outcome is unchanged:
//   * beta == 0 or sign(beta) != sign(M): beta/M > 0 fails; the same for gamma;
//   * |beta| + |gamma| >= |M| (1 + 2^-19) (with |M| in [2^-100, 2^100]): the exact sum of the
//     quotients is at least 1 + 2^-20, so their rounded sum exceeds 1;
//   * tt/M <= 0 while t_min >= 0: t > t_min fails;
//   * |tt| >= fl(|M| t_limit) (1 + 2^-20) with the product normal: the exact quotient exceeds
//     t_limit, so the rounded one is >= t_limit, where t_limit is t_max (any-hit) or
//     min(t_max, closest t) (closest-hit, whose caller rejects t >= closest t).
// The margins cover the at most three roundings in each bound.
__device__ __forceinline__ bool tri_test(const float4 &p0, const float4 &p1, const float4 &p2, const ray_t &r,
                                         float t_limit, float &t_out, float &b_out, float &g_out) {
    const float a = p1.x, b = p1.y, c = p1.z;
    const float d = p2.x, e = p2.y, f = p2.z;
    const float g = r.dx, h = r.dy, i = r.dz;
    const float j = __fsub_rn(p0.x, r.ox()), k = __fsub_rn(p0.y, r.oy()), l = __fsub_rn(p0.z, r.oz());
    float c1 = __fsub_rn(__fmul_rn(e, i), __fmul_rn(h, f));
    float c2 = __fsub_rn(__fmul_rn(g, f), __fmul_rn(d, i));
    float c3 = __fsub_rn(__fmul_rn(d, h), __fmul_rn(e, g));
    const float M = __fadd_rn(__fadd_rn(__fmul_rn(a, c1), __fmul_rn(b, c2)), __fmul_rn(c, c3));
    float beta = __fadd_rn(__fadd_rn(__fmul_rn(j, c1), __fmul_rn(k, c2)), __fmul_rn(l, c3));
    if (beta == 0.f || ((__float_as_uint(beta) ^ __float_as_uint(M)) & 0x80000000u)) return false;
    c1 = __fsub_rn(__fmul_rn(a, k), __fmul_rn(j, b));
    c2 = __fsub_rn(__fmul_rn(j, c), __fmul_rn(a, l));
    c3 = __fsub_rn(__fmul_rn(b, l), __fmul_rn(k, c));
    float gamma = __fadd_rn(__fadd_rn(__fmul_rn(i, c1), __fmul_rn(h, c2)), __fmul_rn(g, c3));
    if (gamma == 0.f || ((__float_as_uint(gamma) ^ __float_as_uint(M)) & 0x80000000u)) return false;
    float tt = -__fadd_rn(__fadd_rn(__fmul_rn(f, c1), __fmul_rn(e, c2)), __fmul_rn(d, c3));
    const float at = signbit(M) ? -tt : tt;  // sign of the quotient tt / M
    if (r.tmin >= 0.f && at <= 0.f) return false;
    const float aM = fabsf(M);
    if (aM >= 0x1p-100f && aM <= 0x1p100f) {
        if (__fadd_rn(fabsf(beta), fabsf(gamma)) >= __fmul_rn(aM, 0x1.00002p0f)) return false;
        if (at > 0.f) {
            if (t_limit <= 0.f) return false;
            const float pl = __fmul_rn(aM, t_limit);
            if (pl >= FLT_MIN && at >= __fmul_rn(pl, 0x1.00001p0f)) return false;
        }
    }
    beta = __fdiv_rn(beta, M);
    gamma = __fdiv_rn(gamma, M);
    tt = __fdiv_rn(tt, M);
    if (tt > r.tmin && tt < r.tmax && beta > 0.f && gamma > 0.f && __fadd_rn(beta, gamma) <= 1.f) {
        t_out = tt;
        b_out = beta;
        g_out = gamma;
        return true;
    }
    return false;
}

// The alpha test of the alpha-aware tracers (rt/cpu/bvh2.cpp:109-117, 168-174): a hit on
// triangle `tri` with material `mat` counts only if diff_geom::opacity() > 0.5
// (libgi/rt.cpp:32-36). The texture coordinate is (1 - beta - gamma) a + beta b + gamma c,
// rounded as diff_geom's constructor rounds it (libgi/rt.cpp:7-14), and the texel is
// texture2d::sample's (libgi/scene.h:28-36): wrap to [0, 1), nearest texel (int)(u w + 0.5),
// index w wrapping to 0. No texture, or a material id beyond the table: opaque. A texel index
// that is not finite (non-finite texture coordinates, undefined in the reference) reads texel 0.
static __device__ __forceinline__ bool alpha_opaque(const alpha_data *A, uint32_t tri, uint32_t mat, float b, float g) {
    if (mat >= A->n_mat) return true;
    const int32_t k = __ldg(A->mat_tex + mat);
    if (k < 0) return true;
    const uint4 t = __ldg(A->tris + tri);
    const float2 ta = __ldg(A->tc + t.x), tb = __ldg(A->tc + t.y), tc = __ldg(A->tc + t.z);
    const float w = __fsub_rn(__fsub_rn(1.0f, b), g);
    float u = __fadd_rn(__fadd_rn(__fmul_rn(w, ta.x), __fmul_rn(b, tb.x)), __fmul_rn(g, tc.x));
    float v = __fadd_rn(__fadd_rn(__fmul_rn(w, ta.y), __fmul_rn(b, tb.y)), __fmul_rn(g, tc.y));
    u = __fsub_rn(u, floorf(u));
    v = __fsub_rn(v, floorf(v));
    const uint4 tx = __ldg(A->tex + k);
    const float fx = __fadd_rn(__fmul_rn(u, (float)tx.x), 0.5f), fy = __fadd_rn(__fmul_rn(v, (float)tx.y), 0.5f);
    int x = isfinite(fx) ? (int)fx : 0, y = isfinite(fy) ? (int)fy : 0;
    if (x == (int)tx.x) x = 0;
    if (y == (int)tx.y) y = 0;
    if (x < 0 || y < 0 || x >= (int)tx.x || y >= (int)tx.y) x = y = 0;
    return __ldg(A->texels + tx.z + (size_t)y * tx.x + x) > 0.5f;
}

// One 256-bit read-only load as four 64-bit words: one child record of a binary node.
__device__ __forceinline__ void ldg256_b64(const float4 *p, uint64_t &a, uint64_t &b, uint64_t &c, uint64_t &d) {
    asm("ld.global.nc.v4.b64 {%0, %1, %2, %3}, [%4];" : "=l"(a), "=l"(b), "=l"(c), "=l"(d) : "l"(p));
}

// Decoding of a leaf child reference: ~ref = (first << 4) | (count - 1).
__device__ __forceinline__ void leaf_range(int32_t ref, uint32_t &first, uint32_t &count) {
    const uint32_t v = ~(uint32_t)ref;
    first = v >> 4;
    count = (v & 15u) + 1u;
}

// Traversal state of one ray, kept in registers; the stack lives in shared memory at
// stk[k * stride] for entry k.
struct trav_t {
    int32_t cur;   // node or leaf reference being processed
    int32_t sp;    // entries on the stack
    uint32_t steps;
    bool done;
    bool found;  // any-hit: an occluder was found
    bool more;     // speculative order: `cur` holds a node or leaf still to visit
    int32_t pend, pend2, pend3;  // speculative order: postponed leaves in visit order (0 = none;
                                 // leaf references are negative)
    uint32_t n_inner, n_tri;  // inner nodes visited and triangles tested (counting kernels only)
    float lim;                // min(t_max, below(hit.t)): a plain ray's closest-hit box limit
    hit_t hit;
};

__device__ __forceinline__ void trav_init(trav_t &s, const dev_scene &sc, const ray_t &r, bool wide = false) {
    s.cur = wide ? sc.root4 : sc.root;
    s.sp = 0;
    s.steps = 0;
    s.done = sc.empty != 0;
    s.found = false;
    s.more = true;
    s.pend = s.pend2 = s.pend3 = 0;
    s.n_inner = 0;
    s.n_tri = 0;
    s.hit.t = FLT_MAX;
    s.lim = fminf(r.tmax, below(FLT_MAX));
    s.hit.b = 0.f;
    s.hit.g = 0.f;
    s.hit.ref = 0u;
    s.hit.rec = 0u;
}

// The test of one child record (layout in bvh_builder.hpp): whether the child is entered (its
// box meets the ray inside [t_min, t_max] and, for closest hits, starts before the closest hit
// so far) and its entry distance. Plain rays take slab2 with the cull folded in; the others the
// reference's compare-and-select form.
template <bool ANY, bool PLAIN>
__device__ __forceinline__ bool child_test(uint64_t xy_lo, uint64_t xy_hi, uint64_t z, const trav_t &s,
                                           const ray_t &r, float &tnear) {
    if (PLAIN) return slab2(xy_lo, xy_hi, z, r, ANY ? r.tmax : s.lim, tnear);
    float lx, ly, hx, hy, lz, hz;
    upk2(xy_lo, lx, ly);
    upk2(xy_hi, hx, hy);
    upk2(z, lz, hz);
    const bool h = slab(lx, ly, lz, hx, hy, hz, r, tnear);
    return ANY ? h : h && tnear < s.hit.t;
}

// Both child tests of the binary node at `np`: entered or not, entry distances, references.
template <bool ANY, bool PLAIN>
__device__ __forceinline__ void node_test(const float4 *np, const trav_t &s, const ray_t &r, bool &hl, bool &hr,
                                          float &dl, float &dr, int32_t &cl, int32_t &cr) {
    uint64_t l0, l1, l2, l3, r0, r1, r2, r3;
    ldg256_b64(np, l0, l1, l2, l3);
    ldg256_b64(np + 2, r0, r1, r2, r3);
    cl = (int32_t)(uint32_t)l3;
    cr = (int32_t)(uint32_t)r3;
    hl = child_test<ANY, PLAIN>(l0, l1, l2, s, r, dl);
    hr = child_test<ANY, PLAIN>(r0, r1, r2, s, r, dr);
}

// One traversal iteration in the while-while order: inner nodes (two box tests each) until the
// ray reaches a leaf or ends, then that leaf's triangle tests. Per ray this is exactly the
// reference's sequence of pops (rt/cpu/bvh2.cpp:82-127 / 147-182): the near child is kept in
// `cur` instead of being pushed and popped straight back, and a leaf is tested when it would
// be popped. Grouping a warp's node visits in one loop and its leaf tests after it keeps the
// lanes on the same code path far more often than one node-or-leaf per iteration would.
template <bool ANY, bool PLAIN, bool COUNT = false, bool ALPHA = false>
__device__ __forceinline__ void trav_iter(trav_t &s, const dev_scene &sc, const ray_t &r, int *stk, int stride, int cap,
                                          unsigned *err) {
    while (s.cur >= 0) {
        if (++s.steps > kStepLimit) {
            atomicOr(err, ERR_STEP_LIMIT);
            s.done = true;
            return;
        }
        if (COUNT) ++s.n_inner;
        float dl, dr;
        bool hl, hr;
        int32_t cl, cr;
        node_test<ANY, PLAIN>(sc.nodes + 4 * (size_t)s.cur, s, r, hl, hr, dl, dr, cl, cr);
        if (hl && hr) {
            const bool left_first = dl < dr;
            if (s.sp >= cap) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                s.done = true;
                return;
            }
            stk[s.sp * stride] = left_first ? cr : cl;
            ++s.sp;
            s.cur = left_first ? cl : cr;
        } else if (hl || hr) {
            s.cur = hl ? cl : cr;
        } else {
            if (s.sp == 0) {
                s.done = true;
                return;
            }
            --s.sp;
            s.cur = stk[s.sp * stride];
        }
    }
    if (++s.steps > kStepLimit) {
        atomicOr(err, ERR_STEP_LIMIT);
        s.done = true;
        return;
    }
    uint32_t first, count;
    leaf_range(s.cur, first, count);
    const float4 *rp = sc.records + 3 * (size_t)first;
    for (uint32_t k = 0; k < count; ++k) {
        if (COUNT) ++s.n_tri;
        const float4 p0 = __ldg(rp + 3 * k), p1 = __ldg(rp + 3 * k + 1), p2 = __ldg(rp + 3 * k + 2);
        float t, b, g;
        if (tri_test(p0, p1, p2, r, ANY ? r.tmax : fminf(r.tmax, s.hit.t), t, b, g) && (ANY || t < s.hit.t) &&
                (!ALPHA || alpha_opaque(sc.alpha, __float_as_uint(p0.w), __float_as_uint(p1.w), b, g))) {
            s.hit.t = t;
            if (!ANY) s.lim = fminf(r.tmax, below(t));
            s.hit.b = b;
            s.hit.g = g;
            s.hit.ref = __float_as_uint(p0.w);
            s.hit.rec = first + k;
            if (ANY) {
                s.found = true;
                s.done = true;
                return;
            }
        }
    }
    if (s.sp == 0) {
        s.done = true;
        return;
    }
    --s.sp;
    s.cur = stk[s.sp * stride];
}

// The if-if order: one inner node or one leaf per call (the reference's if-if tracer,
// rt/cuda/trace-kernels.cu:1058-1149, visits in the same per-ray order as while-while). Lanes of
// a warp at nodes and lanes at leaves take different branches in the same call.
template <bool ANY, bool PLAIN, bool COUNT = false, bool ALPHA = false>
__device__ __forceinline__ void trav_step(trav_t &s, const dev_scene &sc, const ray_t &r, int *stk, int stride, int cap,
                                          unsigned *err) {
    if (++s.steps > kStepLimit) {
        atomicOr(err, ERR_STEP_LIMIT);
        s.done = true;
        return;
    }
    if (s.cur >= 0) {
        if (COUNT) ++s.n_inner;
        float dl, dr;
        bool hl, hr;
        int32_t cl, cr;
        node_test<ANY, PLAIN>(sc.nodes + 4 * (size_t)s.cur, s, r, hl, hr, dl, dr, cl, cr);
        if (hl && hr) {
            const bool left_first = dl < dr;
            if (s.sp >= cap) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                s.done = true;
                return;
            }
            stk[s.sp * stride] = left_first ? cr : cl;
            ++s.sp;
            s.cur = left_first ? cl : cr;
            return;
        }
        if (hl || hr) {
            s.cur = hl ? cl : cr;
            return;
        }
    } else {
        uint32_t first, count;
        leaf_range(s.cur, first, count);
        const float4 *rp = sc.records + 3 * (size_t)first;
        for (uint32_t k = 0; k < count; ++k) {
            if (COUNT) ++s.n_tri;
            const float4 p0 = __ldg(rp + 3 * k), p1 = __ldg(rp + 3 * k + 1), p2 = __ldg(rp + 3 * k + 2);
            float t, b, g;
            if (tri_test(p0, p1, p2, r, ANY ? r.tmax : fminf(r.tmax, s.hit.t), t, b, g) && (ANY || t < s.hit.t) &&
                (!ALPHA || alpha_opaque(sc.alpha, __float_as_uint(p0.w), __float_as_uint(p1.w), b, g))) {
                s.hit.t = t;
                if (!ANY) s.lim = fminf(r.tmax, below(t));
                s.hit.b = b;
                s.hit.g = g;
                s.hit.ref = __float_as_uint(p0.w);
                s.hit.rec = first + k;
                if (ANY) {
                    s.found = true;
                    s.done = true;
                    return;
                }
            }
        }
    }
    if (s.sp == 0) {
        s.done = true;
        return;
    }
    --s.sp;
    s.cur = stk[s.sp * stride];
}

// Inner-node visit shared by the speculative order: box tests of `cur`, then near child,
// push of the far child, or pop. Clears `more` when the stack runs empty.
template <bool ANY, bool PLAIN>
__device__ __forceinline__ void spec_node(trav_t &s, const dev_scene &sc, const ray_t &r, int *stk, int stride, int cap,
                                          unsigned *err) {
    float dl, dr;
    bool hl, hr;
    int32_t cl, cr;
    node_test<ANY, PLAIN>(sc.nodes + 4 * (size_t)s.cur, s, r, hl, hr, dl, dr, cl, cr);
    if (ANY) {
        if (hl && hr) {
            const bool left_first = dl < dr;
            if (s.sp >= cap) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                s.done = true;
                return;
            }
            stk[s.sp * stride] = left_first ? cr : cl;
            ++s.sp;
            s.cur = left_first ? cl : cr;
        } else if (hl || hr) {
            s.cur = hl ? cl : cr;
        } else if (s.sp == 0) {
            s.more = false;
        } else {
            --s.sp;
            s.cur = stk[s.sp * stride];
        }
        return;
    }
    // Closest hit: the same choices with one selection of the near and far child and the pop as
    // a predicated load instead of three branches (on GB300 0.8 % off the fused path loop; the
    // any-hit kernels compiled this way ran 3 % slower, so they keep the branches above).
    // Near child: the left one if only it is entered, or both are and it is nearer (ties right).
    const bool left_first = hl && (!hr || dl < dr);
    const int32_t nearc = left_first ? cl : cr, farc = left_first ? cr : cl;
    if (hl && hr) {
        if (s.sp >= cap) {
            atomicOr(err, ERR_STACK_OVERFLOW);
            s.done = true;
            return;
        }
        stk[s.sp * stride] = farc;
        ++s.sp;
    }
    const bool pop = !hl && !hr && s.sp > 0;
    s.sp -= pop ? 1 : 0;
    const int32_t popped = pop ? stk[s.sp * stride] : nearc;
    s.more = s.more && (hl || hr || pop);  // no child entered and nothing stacked: the search ends
    s.cur = (hl || hr) ? nearc : popped;
}

// Visit of a 4-wide node: four slab tests, the hit children ordered by entry distance (a
// five-comparator sorting network), the nearest kept in `cur` and the others pushed farthest
// first. Every child box is a subset of the binary box the collapse skipped, and rounding is
// monotone, so a child the reference would reach is never culled here.
template <bool ANY, bool PLAIN>
__device__ __forceinline__ void spec_node4(trav_t &s, const dev_scene &sc, const ray_t &r, int *stk, int stride, int cap,
                                           unsigned *err) {
    const float4 *np = sc.nodes4 + 8 * (size_t)s.cur;
    float k[4];
    int c[4];
    bool hit[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        uint64_t xy_lo, xy_hi, z, ref;
        ldg256_b64(np + 2 * i, xy_lo, xy_hi, z, ref);
        c[i] = (int32_t)(uint32_t)ref;
        hit[i] = child_test<ANY, PLAIN>(xy_lo, xy_hi, z, s, r, k[i]);
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        if (!hit[i] || c[i] == kEmptyWideChild) {
            c[i] = kEmptyWideChild;
            k[i] = __int_as_float(0x7f800000);  // +inf
        }
    }
#define GRT_CSWAP(a, b)                          \
    if (k[b] < k[a]) {                           \
        const float tk = k[a];                   \
        k[a] = k[b];                             \
        k[b] = tk;                               \
        const int tc = c[a];                     \
        c[a] = c[b];                             \
        c[b] = tc;                               \
    }
    GRT_CSWAP(0, 1)
    GRT_CSWAP(2, 3)
    GRT_CSWAP(0, 2)
    GRT_CSWAP(1, 3)
    GRT_CSWAP(1, 2)
#undef GRT_CSWAP
    int32_t next = kEmptyWideChild;
#pragma unroll
    for (int i = 3; i >= 0; --i) {
        if (c[i] == kEmptyWideChild) continue;
        if (next != kEmptyWideChild) {
            if (s.sp >= cap) {
                atomicOr(err, ERR_STACK_OVERFLOW);
                s.done = true;
                return;
            }
            stk[s.sp * stride] = next;
            ++s.sp;
        }
        next = c[i];
    }
    if (next != kEmptyWideChild) {
        s.cur = next;
    } else if (s.sp == 0) {
        s.more = false;
    } else {
        --s.sp;
        s.cur = stk[s.sp * stride];
    }
}

// The speculative while-while order (the reference's speculativewhilewhile_traversal,
// rt/cuda/trace-kernels.cu:1433-1540, after Aila and Laine): a lane that reaches a leaf
// postpones it and keeps visiting inner nodes while other lanes of the warp are still looking
// for their first leaf; then all postponed leaves are tested together. The reference postpones
// one leaf; here a lane may postpone up to cfg.pend (1 to 3) before the leaf phase, so that lanes
// already holding a leaf do useful work instead of idling while the warp searches (on GB300 two
// took 9 % off the fused path step and three 14 % off fused direct lighting). The warp leaves
// the node phase once at most cfg.exit lanes are still searching for their first leaf; those lanes
// resume where they stopped in the next call, so this changes when leaves are tested, not which
// (leaving with up to 6 to 8 of 32 lanes still searching took another 5 % off the fused path
// step). The three parameters (cfg: postponed leaves, exit count, node visits per vote) and the
// stack capacity `cap` are launch arguments, chosen per kernel family and by the autotuner.
// Every lane of the warp must call this together (it ballots over the full warp); `active`
// marks lanes with a ray.
// Each ray's leaves are still tested in the reference's order, but node tests after a
// postponed leaf use the closest hit from before that leaf, so the ray may visit nodes the
// reference would have culled. A triangle found there can replace the reference's answer only
// if its t lies within rounding of the culled box's entry distance: a near-tie.
// ALL_PLAIN: the caller has checked that every active lane's ray is plain, so the node visits
// take the packed slab test without a per-lane choice (half the code of the unrolled visits).
template <bool ANY, bool COUNT, bool WIDE = false, bool ALPHA = false, int VISITS = 0, int PEND = 0,
          bool ALL_PLAIN = false>
__device__ __forceinline__ void trav_spec_iter(trav_t &s, bool active, bool plain, const dev_scene &sc,
                                               const ray_t &r, int *stk, int stride, int cap, const spec_cfg &cfg,
                                               unsigned *err) {
    const bool mine = active && !s.done;
    // VISITS / PEND > 0: instances for the common values, whose loop the compiler unrolls and
    // whose unused postponement slots it drops; 0: the values of `cfg`.
    const int pend = PEND > 0 ? PEND : cfg.pend;
    // One node visit (or postponement of a reached leaf) of this lane, if it has one to make.
    auto visit = [&]() {
        if (mine && !s.done && s.more && s.cur >= 0) {
            if (COUNT) ++s.n_inner;
            if (WIDE) {
                if (ALL_PLAIN || plain)
                    spec_node4<ANY, true>(s, sc, r, stk, stride, cap, err);
                else
                    spec_node4<ANY, false>(s, sc, r, stk, stride, cap, err);
            } else {
                if (ALL_PLAIN || plain)
                    spec_node<ANY, true>(s, sc, r, stk, stride, cap, err);
                else
                    spec_node<ANY, false>(s, sc, r, stk, stride, cap, err);
            }
        }
        const bool slot = pend <= 1 ? s.pend == 0 : pend == 2 ? s.pend2 == 0 : s.pend3 == 0;
        if (mine && !s.done && s.more && s.cur < 0 && slot) {
            // postpone the leaf into the first free slot and go on with the next node
            if (s.pend == 0)
                s.pend = s.cur;
            else if (pend == 2 || s.pend2 == 0)
                s.pend2 = s.cur;
            else
                s.pend3 = s.cur;
            if (s.sp == 0) {
                s.more = false;
            } else {
                --s.sp;
                s.cur = stk[s.sp * stride];
            }
        }
    };
    // cfg.visits node visits per warp vote (three measured on GB300 4.4 % faster than one visit
    // per vote, and 1.2 % faster than two); a lane that has stopped searching may make up to
    // cfg.visits - 1 more speculative node visits before the leaf phase, which leaves its hit within
    // the near-tie class. The warp's visit slots of this call are added to every live lane's step count (an
    // upper bound of its own visits), so the work of a ray on a malformed tree stays bounded
    // across calls, without a per-visit count.
    // At least one visit per vote: every pass then moves each searching lane on by a node or a
    // postponed leaf, so the loop ends (and `slots` reaches the step limit on a malformed tree).
    const int visits = VISITS > 0 ? VISITS : (cfg.visits > 0 ? cfg.visits : 1);
    uint32_t slots = 0;
    for (;;) {
        if (ANY) {  // any hit: a loop (measured faster than the unrolled visits)
#pragma unroll 1
            for (int v = 0; v < (VISITS > 0 ? VISITS : visits); ++v) visit();
        } else {
#pragma unroll
            for (int v = 0; v < (VISITS > 0 ? VISITS : visits); ++v) visit();
        }
        slots += (uint32_t)visits;
        const bool searching = mine && !s.done && s.more && s.pend == 0;
        if (__popc(__ballot_sync(0xffffffffu, searching)) <= cfg.exit || slots >= kStepLimit) break;
    }
    if (mine && !s.done) {
        s.steps += slots;
        if (s.steps > kStepLimit) {
            atomicOr(err, ERR_STEP_LIMIT);
            s.done = true;
        }
    }
    if (mine && !s.done) {
        while (s.pend != 0 && !s.done) {
            uint32_t first, count;
            leaf_range(s.pend, first, count);
            s.pend = s.pend2;  // slots beyond the postponing limit stay 0
            s.pend2 = s.pend3;
            s.pend3 = 0;
            ++s.steps;
            const float4 *rp = sc.records + 3 * (size_t)first;
            for (uint32_t k = 0; k < count; ++k) {
                if (COUNT) ++s.n_tri;
                const float4 p0 = __ldg(rp + 3 * k), p1 = __ldg(rp + 3 * k + 1), p2 = __ldg(rp + 3 * k + 2);
                float t, b, g;
                if (tri_test(p0, p1, p2, r, ANY ? r.tmax : fminf(r.tmax, s.hit.t), t, b, g) && (ANY || t < s.hit.t) &&
                (!ALPHA || alpha_opaque(sc.alpha, __float_as_uint(p0.w), __float_as_uint(p1.w), b, g))) {
                    s.hit.t = t;
                    if (!ANY) s.lim = fminf(r.tmax, below(t));
                    s.hit.b = b;
                    s.hit.g = g;
                    s.hit.ref = __float_as_uint(p0.w);
                    s.hit.rec = first + k;
                    if (ANY) {
                        s.found = true;
                        s.done = true;
                        break;
                    }
                }
            }
        }
        if (!s.done && !s.more && s.pend == 0) s.done = true;
    }
}

// One iteration of a non-speculative loop order for this lane's ray (PLAIN: min/max slab test,
// see ray_is_plain). The speculative order is trav_spec_iter, which the whole warp calls together.
template <int ORDER, bool ANY, bool COUNT, bool PLAIN, bool ALPHA = false>
__device__ __forceinline__ void trav_advance(trav_t &s, const dev_scene &sc, const ray_t &r, int *stk, int stride,
                                             int cap, unsigned *err) {
    if (ORDER == WHILE_WHILE)
        trav_iter<ANY, PLAIN, COUNT, ALPHA>(s, sc, r, stk, stride, cap, err);
    else
        trav_step<ANY, PLAIN, COUNT, ALPHA>(s, sc, r, stk, stride, cap, err);
}

// Writes one result in the reference's encodings (see include/grt.h).
template <bool ANY>
__device__ __forceinline__ void store_hit(grt_hit *hits, uint32_t i, const trav_t &s) {
    if (ANY) {
        hits[i].t = s.found ? 4294967296.0f : FLT_MAX;
        hits[i].ref = s.found ? 0xFFFFFFFFu : 0u;
    } else {
        reinterpret_cast<float4 *>(hits)[i] = make_float4(s.hit.t, s.hit.b, s.hit.g, __uint_as_float(s.hit.ref));
    }
}

}  // namespace grt
