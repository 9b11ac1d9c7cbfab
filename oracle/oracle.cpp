// ORACLE — test infrastructure only. Never linked into, loaded by or called from the product.
//
// A CPU restatement of the reference's ray-traversal path (lwolf98/illum-rt, "RTGI"):
//   * BVH construction: bvh_ctor::build + early split clipping + the OM / SM / SAH subdivision
//     (rt/cpu/bvh-ctor.h:96-503), indexed triangle layout as the CUDA platform uses it
//     (rt/cuda/base.cpp:88-117);
//   * ray/box and ray/triangle tests (libgi/intersect.h:19-74, 230-267);
//   * binary_bvh_tracer::closest_hit / any_hit (rt/cpu/bvh2.cpp:71-189);
//   * the OpenMP batch loop of the CPU platform (rt/cpu/wavefront.cpp:53-70).
// It is written in C++ rather than C because the reference's builder orders primitives with
// std::sort, whose placement of equal keys is part of the result; calling the same library
// routine with the same comparator reproduces it. Compiled with -ffp-contract=off so every
// float operation rounds exactly as written, on x86-64 and aarch64 alike.
//
// Pinning: tests compare this restatement with the reference itself (oracle/_ref, built from
// the reference sources by oracle/build_ref.sh where they are available) node for node, and
// with golden fixtures generated from oracle/_ref (tests/golden/).
//
// One deliberate difference: the reference traversal keeps a fixed 25-entry stack
// (rt/cpu/bvh2.cpp:76,145) and overflows it on trees deeper than 24. The restatement uses a
// growable stack and reports the deepest stack it needed, so callers can flag rays on which
// the reference itself would have had undefined behaviour.
#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <omp.h>
#include <vector>

namespace orc {

struct v3 {
    float x, y, z;
    float operator[](int k) const { return k == 0 ? x : (k == 1 ? y : z); }
};

// aabb with the reference's grow semantics (libgi/intersect.h:5-16, glm::min/max semantics:
// min(x, y) = (y < x) ? y : x, max(x, y) = (x < y) ? y : x).
struct box {
    v3 lo{FLT_MAX, FLT_MAX, FLT_MAX}, hi{-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void grow(const v3 &v) {
        lo = {(lo.x < v.x) ? lo.x : v.x, (lo.y < v.y) ? lo.y : v.y, (lo.z < v.z) ? lo.z : v.z};
        hi = {(v.x < hi.x) ? hi.x : v.x, (v.y < hi.y) ? hi.y : v.y, (v.z < hi.z) ? hi.z : v.z};
    }
    void grow(const box &o) {
        lo = {(lo.x < o.lo.x) ? lo.x : o.lo.x, (lo.y < o.lo.y) ? lo.y : o.lo.y, (lo.z < o.lo.z) ? lo.z : o.lo.z};
        hi = {(o.hi.x < hi.x) ? hi.x : o.hi.x, (o.hi.y < hi.y) ? hi.y : o.hi.y, (o.hi.z < hi.z) ? hi.z : o.hi.z};
    }
    v3 center() const { return {(lo.x + hi.x) * 0.5f, (lo.y + hi.y) * 0.5f, (lo.z + hi.z) * 0.5f}; }
    v3 extent() const { return {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z}; }
};

// surface area as written in bvh-ctor.h:121-124, 184-187, 387-390
inline float area(const box &b) {
    v3 e = b.extent();
    return 2 * (e.x * e.y + e.x * e.z + e.y * e.z);
}

inline float fmax_ref(float a, float b) { return (a < b) ? b : a; }  // std::max
inline int largest_axis(const v3 &e) {
    float largest = fmax_ref(e.x, fmax_ref(e.y, e.z));
    return largest == e.x ? 0 : (largest == e.y ? 1 : 2);
}

// bbvh_node (rt/cpu/bvh.h:42-52): a leaf has link_l = -offset, link_r = -count.
struct node {
    box l, r;
    int32_t link_l = 0, link_r = 0;
    bool inner() const { return link_r >= 0; }
};

struct prim {
    box b;
    uint32_t tri;
};

struct scene {
    const float *v4;
    const uint32_t *t4;
    uint32_t nv, nt;
    v3 vert(uint32_t i) const { return {v4[4 * i], v4[4 * i + 1], v4[4 * i + 2]}; }
};

struct builder {
    const scene &sc;
    int split_type;  // 0 om, 1 sm, 2 sah
    int max_tris, planes;
    bool esc;
    std::vector<prim> prims;
    std::vector<uint32_t> index;
    std::vector<node> nodes;
    bool failed = false;

    builder(const scene &s, int type, int mt, int np, bool e) : sc(s), split_type(type), max_tris(mt), planes(np), esc(e) {}

    float c(uint32_t pi, int axis) const { return prims[pi].b.center()[axis]; }
    void sort_range(uint32_t start, uint32_t end, int axis) {
        std::sort(index.data() + start, index.data() + end,
                  [&](uint32_t a, uint32_t b) { return c(a, axis) < c(b, axis); });
    }
    box range_box(uint32_t start, uint32_t end) const {
        box b;
        for (uint32_t i = start; i < end; ++i) b.grow(prims[index[i]].b);
        return b;
    }
    uint32_t make_leaf(uint32_t start, uint32_t end) {
        uint32_t id = (uint32_t)nodes.size();
        nodes.emplace_back();
        nodes[id].link_l = -(int32_t)start;
        nodes[id].link_r = -(int32_t)(end - start);
        return id;
    }

    // Split of one polygon at the centre of its largest box axis until each part's box area is
    // at most `thres` (the split() helper, rt/cpu/bvh-ctor.h:120-179).
    void split_poly(const std::vector<v3> &poly, float thres, std::vector<box> &out) {
        box b;
        for (const v3 &v : poly) b.grow(v);
        if (area(b) <= thres) {
            out.push_back(b);
            return;
        }
        int ax = largest_axis(b.extent());
        float center = (b.hi[ax] + b.lo[ax]) * 0.5f;
        int n = (int)poly.size();
        bool last_left = poly[0][ax] < center;
        int cross_first = -1, cross_second = -1;
        for (int i = 0; i < n; ++i) {
            bool left = poly[i][ax] < center;
            if (left != last_left) {
                if (cross_first == -1)
                    cross_first = i - 1;
                else
                    cross_second = i - 1;
            }
            last_left = left;
        }
        if (cross_second == -1) cross_second = n - 1;
        if (cross_first == -1) {  // unreachable for finite input (the reference asserts here)
            out.push_back(b);
            return;
        }
        auto ipoint = [&](int a) {
            float delta = center - poly[a][ax];
            int bb = a + 1 < n ? a + 1 : 0;
            float s = delta / (poly[bb][ax] - poly[a][ax]);
            return v3{poly[a].x + (poly[bb].x - poly[a].x) * s, poly[a].y + (poly[bb].y - poly[a].y) * s,
                      poly[a].z + (poly[bb].z - poly[a].z) * s};
        };
        v3 c1 = ipoint(cross_first), c2 = ipoint(cross_second);
        std::vector<v3> p1, p2;
        for (int i = 0; i <= cross_first; ++i) p1.push_back(poly[i]);
        p1.push_back(c1);
        p2.push_back(c1);
        for (int i = cross_first + 1; i <= cross_second; ++i) p2.push_back(poly[i]);
        p2.push_back(c2);
        p1.push_back(c2);
        for (int i = cross_second + 1; i < n; ++i) p1.push_back(poly[i]);
        auto same = [](const v3 &a, const v3 &b) { return a.x == b.x && a.y == b.y && a.z == b.z; };
        p1.erase(std::unique(p1.begin(), p1.end(), same), p1.end());
        p2.erase(std::unique(p2.begin(), p2.end(), same), p2.end());
        split_poly(p1, thres, out);
        split_poly(p2, thres, out);
    }

    // early_split_clipping (rt/cpu/bvh-ctor.h:181-226): threshold = area at the 90th percentile.
    void early_split_clipping() {
        std::vector<float> areas(prims.size());
        for (size_t i = 0; i < prims.size(); ++i) areas[i] = area(prims[i].b);
        size_t k = 9 * prims.size() / 10;
        std::nth_element(areas.begin(), areas.begin() + k, areas.end());
        float thres = areas[k];
        uint32_t N = (uint32_t)prims.size();
        std::vector<box> gen;
        for (uint32_t i = 0; i < N; ++i) {
            const uint32_t *t = sc.t4 + 4 * index[i];
            std::vector<v3> poly = {sc.vert(t[0]), sc.vert(t[1]), sc.vert(t[2])};
            gen.clear();
            split_poly(poly, thres, gen);
            prims[i] = {gen[0], i};
            for (size_t j = 1; j < gen.size(); ++j) {
                prims.push_back({gen[j], i});
                index.push_back((uint32_t)prims.size() - 1);
            }
        }
    }

    // Object median (rt/cpu/bvh-ctor.h:251-300).
    uint32_t subdivide_om(uint32_t start, uint32_t end) {
        if (end - start <= (uint32_t)max_tris) return make_leaf(start, end);
        box b = range_box(start, end);
        sort_range(start, end, largest_axis(b.extent()));
        uint32_t mid = start + (end - start) / 2;
        uint32_t id = (uint32_t)nodes.size();
        nodes.emplace_back();
        uint32_t l = subdivide(start, mid);
        uint32_t r = subdivide(mid, end);
        nodes[id].link_l = (int32_t)l;
        nodes[id].link_r = (int32_t)r;
        nodes[id].l = range_box(start, mid);
        nodes[id].r = range_box(mid, end);
        return id;
    }

    // Partition of index[start, end) by center <= plane, as both the spatial-median and the SAH
    // builders do it (rt/cpu/bvh-ctor.h:333-343, 427-440). Returns the resulting mid.
    uint32_t partition(uint32_t start, uint32_t end, int ax, float plane) {
        uint32_t mid = start;
        uint32_t *L = index.data() + start, *R = index.data() + end - 1;
        while (L < R) {
            while (c(*L, ax) <= plane && L < R) {
                ++L;
                ++mid;
            }
            while (c(*R, ax) > plane && L < R) --R;
            if (c(*L, ax) > c(*R, ax) && L < R) std::swap(*L, *R);
        }
        return mid;
    }

    // Spatial median (rt/cpu/bvh-ctor.h:302-369).
    uint32_t subdivide_sm(uint32_t start, uint32_t end) {
        if (end - start <= (uint32_t)max_tris) return make_leaf(start, end);
        box b = range_box(start, end);
        v3 e = b.extent();
        int ax = largest_axis(e);
        v3 half = {b.lo.x + e.x * 0.5f, b.lo.y + e.y * 0.5f, b.lo.z + e.z * 0.5f};
        uint32_t mid = partition(start, end, ax, half[ax]);
        if (mid == start || mid == end - 1) {
            sort_range(start, end, ax);
            mid = start + (end - start) / 2;
        }
        uint32_t id = (uint32_t)nodes.size();
        nodes.emplace_back();
        uint32_t l = subdivide(start, mid);
        uint32_t r = subdivide(mid, end);
        nodes[id].link_l = (int32_t)l;
        nodes[id].link_r = (int32_t)r;
        nodes[id].l = range_box(start, mid);
        nodes[id].r = range_box(mid, end);
        return id;
    }

    // SAH over `planes` uniform planes on the largest axis (rt/cpu/bvh-ctor.h:371-503).
    uint32_t subdivide_sah(uint32_t start, uint32_t end) {
        if (end - start <= (uint32_t)max_tris) return make_leaf(start, end);
        box b = range_box(start, end);
        float surf = area(b);
        v3 e = b.extent();
        int ax = largest_axis(e);
        uint32_t mid = start;
        box bl, br;
        if (surf == 0) {
            sort_range(start, end, ax);
            mid = start + (end - start) / 2;
            bl = range_box(start, mid);
            br = range_box(mid, end);
        } else {
            float cost_l = FLT_MAX, cost_r = FLT_MAX;
            bool use_om = true;
            auto try_plane = [&](float plane) {
                uint32_t cur = partition(start, end, ax, plane);
                if (cur == start || cur == end - 1) {
                    if (!use_om) return;
                    sort_range(start, end, ax);
                    cur = start + (end - start) / 2;
                    use_om = false;
                }
                box cbl = range_box(start, cur), cbr = range_box(cur, end);
                float cl = (area(cbl) / surf) * (float)(int)(cur - start);
                float cr = (area(cbr) / surf) * (float)(int)(end - cur);
                if (cl + cr < cost_l + cost_r) {
                    bl = cbl;
                    br = cbr;
                    cost_l = cl;
                    cost_r = cr;
                    mid = cur;
                }
            };
            int np = planes;
            if ((int)(end - start) < np) np = (int)(end - start);
            for (int i = 0; i < np; ++i) try_plane(b.lo[ax] + (float)(i + 1) * (e[ax] / (float)(np + 1)));
            const float K_T = 1, K_I = 1;
            if (max_tris > 1 && (K_I * (float)(int)(end - start)) < (K_T + K_I * (cost_l + cost_r)) &&
                (int)(end - start) <= max_tris)
                return make_leaf(start, end);  // unreachable: ranges this small returned above
        }
        if (mid == start || mid == end) {  // no split found; the reference would recurse forever
            failed = true;
            return make_leaf(start, end);
        }
        uint32_t id = (uint32_t)nodes.size();
        nodes.emplace_back();
        uint32_t l = subdivide(start, mid);
        uint32_t r = subdivide(mid, end);
        nodes[id].link_l = (int32_t)l;
        nodes[id].link_r = (int32_t)r;
        nodes[id].l = bl;
        nodes[id].r = br;
        return id;
    }

    uint32_t subdivide(uint32_t start, uint32_t end) {
        if (failed) return make_leaf(start, end);
        switch (split_type) {
            case 0: return subdivide_om(start, end);
            case 1: return subdivide_sm(start, end);
            default: return subdivide_sah(start, end);
        }
    }

    // bvh_ctor::build + commit_shuffled_triangles for the indexed layout (bvh-ctor.h:96-118, 239-248)
    uint32_t build() {
        prims.resize(sc.nt);
        index.resize(sc.nt);
        for (uint32_t i = 0; i < sc.nt; ++i) {
            const uint32_t *t = sc.t4 + 4 * i;
            box b;
            b.grow(sc.vert(t[0]));
            b.grow(sc.vert(t[1]));
            b.grow(sc.vert(t[2]));
            prims[i] = {b, i};
            index[i] = i;
        }
        if (esc && sc.nt > 0) early_split_clipping();
        uint32_t root = subdivide(0, (uint32_t)prims.size());
        if (esc)
            for (auto &x : index) x = prims[x].tri;
        return root;
    }
};

// Texture data of the alpha-aware tracers: a texture coordinate per vertex, a texture per
// material (or none) and single-channel alpha textures of w x h texels, row by row.
struct alpha_set {
    bool on = false;
    std::vector<float> tc;          // 2 per vertex
    std::vector<int32_t> mat_tex;   // texture index per material, -1 for none
    std::vector<uint32_t> w, h, off;
    std::vector<float> texels;
};

struct bvh {
    scene sc;
    std::vector<float> v4;
    std::vector<uint32_t> t4;
    uint32_t root = 0;
    std::vector<node> nodes;
    std::vector<uint32_t> index;
    bool failed = false;
    alpha_set alpha;
};

struct ray {
    v3 o, d, id;
    float tmin, tmax;
};

inline ray load_ray(const float *r) {
    ray out;
    out.o = {r[0], r[1], r[2]};
    out.d = {r[4], r[5], r[6]};
    out.id = {1.0f / r[4], 1.0f / r[5], 1.0f / r[6]};  // ray::ray (libgi/rt.h:28)
    out.tmin = r[3];
    out.tmax = r[7];
    return out;
}

struct hit {
    float t = FLT_MAX, beta = 0, gamma = 0;
    uint32_t ref = 0;
};

// Cramer's rule ray/triangle test (libgi/intersect.h:19-74), same operation order.
inline bool intersect_tri(const scene &sc, uint32_t tri, const ray &r, hit &info) {
    const uint32_t *t = sc.t4 + 4 * tri;
    v3 A = sc.vert(t[0]), B = sc.vert(t[1]), C = sc.vert(t[2]);
    const float a = A.x - B.x, b = A.y - B.y, c = A.z - B.z;
    const float d = A.x - C.x, e = A.y - C.y, f = A.z - C.z;
    const float g = r.d.x, h = r.d.y, i = r.d.z;
    const float j = A.x - r.o.x, k = A.y - r.o.y, l = A.z - r.o.z;
    float common1 = e * i - h * f;
    float common2 = g * f - d * i;
    float common3 = d * h - e * g;
    float M = a * common1 + b * common2 + c * common3;
    float beta = j * common1 + k * common2 + l * common3;
    common1 = a * k - j * b;
    common2 = j * c - a * l;
    common3 = b * l - k * c;
    float gamma = i * common1 + h * common2 + g * common3;
    float tt = -(f * common1 + e * common2 + d * common3);
    beta /= M;
    gamma /= M;
    tt /= M;
    if (tt > r.tmin && tt < r.tmax)
        if (beta > 0 && gamma > 0 && beta + gamma <= 1) {
            info.t = tt;
            info.beta = beta;
            info.gamma = gamma;
            return true;
        }
    return false;
}

// Slab test intersect4 (libgi/intersect.h:230-267), same selects so NaN cases match too.
inline bool intersect_box(const box &bx, const ray &r, float &is) {
    float t1x_tmp = (bx.lo.x - r.o.x) * r.id.x;
    float t2x_tmp = (bx.hi.x - r.o.x) * r.id.x;
    float t1x = (t1x_tmp < t2x_tmp) ? t1x_tmp : t2x_tmp;
    float t2x = (t2x_tmp < t1x_tmp) ? t1x_tmp : t2x_tmp;
    float t1y_tmp = (bx.lo.y - r.o.y) * r.id.y;
    float t2y_tmp = (bx.hi.y - r.o.y) * r.id.y;
    float t1y = (t1y_tmp < t2y_tmp) ? t1y_tmp : t2y_tmp;
    float t2y = (t2y_tmp < t1y_tmp) ? t1y_tmp : t2y_tmp;
    float t1z_tmp = (bx.lo.z - r.o.z) * r.id.z;
    float t2z_tmp = (bx.hi.z - r.o.z) * r.id.z;
    float t1z = (t1z_tmp < t2z_tmp) ? t1z_tmp : t2z_tmp;
    float t2z = (t2z_tmp < t1z_tmp) ? t1z_tmp : t2z_tmp;
    float t1 = (t1x < t1y) ? t1y : t1x;
    t1 = (t1z < t1) ? t1 : t1z;
    float t2 = (t2x < t2y) ? t2x : t2y;
    t2 = (t2z < t2) ? t2z : t2;
    if (t1 > t2) return false;
    if (t2 < r.tmin) return false;
    if (t1 > r.tmax) return false;
    is = t1;
    return true;
}

struct counters {
    uint32_t inner = 0, tris = 0, max_sp = 0;
};

// The alpha test of the alpha-aware tracers (rt/cpu/bvh2.cpp:109-117, 168-174): a hit counts only
// if diff_geom::opacity() > 0.5 (libgi/rt.cpp:32-36). The texture coordinate is interpolated as in
// diff_geom's constructor, (1 - beta - gamma) a + beta b + gamma c (libgi/rt.cpp:7-14), and
// looked up by texture2d::sample (libgi/scene.h:28-36): wrap to [0, 1), nearest texel by
// (int)(u w + 0.5), index w wrapping to 0. A material without a texture is opaque. Material ids
// beyond the table, and texture coordinates whose texel index is not finite, are outside what
// the reference defines; here they count as opaque and as texel 0.
inline bool opaque(const bvh &h, uint32_t tri, const hit &is) {
    const alpha_set &A = h.alpha;
    const uint32_t *t = h.sc.t4 + 4 * tri;
    const uint32_t m = t[3];
    if (m >= A.mat_tex.size() || A.mat_tex[m] < 0) return true;
    const uint32_t k = (uint32_t)A.mat_tex[m];
    const float w = 1.0f - is.beta - is.gamma;
    const float *a = A.tc.data() + 2 * t[0], *b = A.tc.data() + 2 * t[1], *c = A.tc.data() + 2 * t[2];
    float u = w * a[0] + is.beta * b[0] + is.gamma * c[0];
    float v = w * a[1] + is.beta * b[1] + is.gamma * c[1];
    u = u - std::floor(u);
    v = v - std::floor(v);
    const float fx = u * (float)A.w[k] + 0.5f, fy = v * (float)A.h[k] + 0.5f;
    int x = std::isfinite(fx) ? (int)fx : 0, y = std::isfinite(fy) ? (int)fy : 0;
    if (x == (int)A.w[k]) x = 0;
    if (y == (int)A.h[k]) y = 0;
    if (x < 0 || y < 0 || x >= (int)A.w[k] || y >= (int)A.h[k]) x = y = 0;
    return A.texels[A.off[k] + (size_t)y * A.w[k] + x] > 0.5f;
}

// binary_bvh_tracer::closest_hit (rt/cpu/bvh2.cpp:71-137), non-alpha, indexed layout.
inline hit closest_hit(const bvh &h, const ray &r, counters *cnt) {
    hit closest, is;
    uint32_t stack_local[64];
    std::vector<uint32_t> stack_big;
    uint32_t *stack = stack_local;
    uint32_t cap = 64;
    int32_t sp = 0;
    stack[0] = h.root;
    uint32_t max_sp = 0;
    auto push = [&](uint32_t v) {
        ++sp;
        if ((uint32_t)sp >= cap) {
            if (stack_big.empty()) stack_big.assign(stack_local, stack_local + cap);
            stack_big.resize(cap * 2);
            cap *= 2;
            stack = stack_big.data();
        }
        stack[sp] = v;
        if ((uint32_t)sp > max_sp) max_sp = sp;
    };
    uint32_t n_inner = 0, n_tri = 0;
    while (sp >= 0) {
        const node &n = h.nodes[stack[sp--]];
        if (n.inner()) {
            ++n_inner;
            float dl, dr;
            bool hl = intersect_box(n.l, r, dl) && dl < closest.t;
            bool hr = intersect_box(n.r, r, dr) && dr < closest.t;
            if (hl && hr) {
                if (dl < dr) {
                    push(n.link_r);
                    push(n.link_l);
                } else {
                    push(n.link_l);
                    push(n.link_r);
                }
            } else if (hl)
                push(n.link_l);
            else if (hr)
                push(n.link_r);
        } else {
            int32_t off = -n.link_l, count = -n.link_r;
            for (int32_t i = 0; i < count; ++i) {
                uint32_t tri = h.index[off + i];
                ++n_tri;
                if (intersect_tri(h.sc, tri, r, is)) {
                    if (h.alpha.on && !opaque(h, tri, is)) continue;
                    if (is.t < closest.t) {
                        closest = is;
                        closest.ref = tri;
                    }
                }
            }
        }
    }
    if (cnt) *cnt = {n_inner, n_tri, max_sp};
    return closest;
}

// binary_bvh_tracer::any_hit (rt/cpu/bvh2.cpp:139-189), non-alpha, indexed layout.
inline bool any_hit(const bvh &h, const ray &r, counters *cnt) {
    hit is;
    std::vector<uint32_t> stack(64);
    int32_t sp = 0;
    stack[0] = h.root;
    uint32_t max_sp = 0, n_inner = 0, n_tri = 0;
    auto push = [&](uint32_t v) {
        ++sp;
        if ((size_t)sp >= stack.size()) stack.resize(stack.size() * 2);
        stack[sp] = v;
        if ((uint32_t)sp > max_sp) max_sp = sp;
    };
    bool result = false;
    while (sp >= 0 && !result) {
        const node &n = h.nodes[stack[sp--]];
        if (n.inner()) {
            ++n_inner;
            float dl, dr;
            bool hl = intersect_box(n.l, r, dl);
            bool hr = intersect_box(n.r, r, dr);
            if (hl && hr) {
                if (dl < dr) {
                    push(n.link_r);
                    push(n.link_l);
                } else {
                    push(n.link_l);
                    push(n.link_r);
                }
            } else if (hl)
                push(n.link_l);
            else if (hr)
                push(n.link_r);
        } else {
            int32_t off = -n.link_l, count = -n.link_r;
            for (int32_t i = 0; i < count; ++i) {
                ++n_tri;
                if (intersect_tri(h.sc, h.index[off + i], r, is)) {
                    if (h.alpha.on && !opaque(h, h.index[off + i], is)) continue;
                    result = true;
                    break;
                }
            }
        }
    }
    if (cnt) *cnt = {n_inner, n_tri, max_sp};
    return result;
}

inline void set_threads(int threads) {
    if (threads > 0) omp_set_num_threads(threads);
}


// ---- ray generation around the traversal --------------------------------------------------
//
// Restatement, for checking, of the product's bounce and shadow-ray definitions: PCG32
// (libgi/random.h:59-96), cosine_sample_hemisphere / uniform_sample_disk
// (libgi/sampling.h:13-17, 32-36) with sin/cos of 2*pi*u from the Taylor polynomials of the
// remaining quarter-turn angle, align (libgi/util.h:212-218), flip_normals_to_ray
// (libgi/util.h:221-225), and length_exclusive (libgi/rt.h:30). Plain float arithmetic; the
// file is compiled with -ffp-contract=off so each operation rounds as written.

struct rng32 {
    uint64_t state = 0, inc = 1;
    uint32_t next() {
        uint64_t old = state;
        state = old * 0x5851f42d4c957f2dULL + inc;
        uint32_t x = (uint32_t)(((old >> 18u) ^ old) >> 27u);
        uint32_t rot = (uint32_t)(old >> 59u);
        return (x >> rot) | (x << ((~rot + 1u) & 31u));
    }
    void seq(uint64_t s) {
        state = 0u;
        inc = (s << 1u) | 1u;
        next();
        state += 0x853c49e6748fea9bULL;
        next();
    }
    float uniform() {
        float f = (float)next() * 0x1p-32f;
        return f < 0x1.fffffep-1f ? f : 0x1.fffffep-1f;
    }
};

inline void turn_sincos(float u, float &s, float &c) {
    float t4 = u * 4.0f;
    int q = (int)t4;
    float x = (t4 - (float)q) * 0x1.921fb6p+0f;
    float x2 = x * x;
    const float sc[7] = {0x1.612462p-33f, -0x1.ae6456p-26f, 0x1.71de3ap-19f, -0x1.a01a02p-13f,
                         0x1.111112p-7f, -0x1.555556p-3f, 1.0f};
    const float cc[7] = {0x1.1eed8ep-29f, -0x1.27e4fcp-22f, 0x1.a01a02p-16f, -0x1.6c16c2p-10f,
                         0x1.555556p-5f, -0.5f, 1.0f};
    float ps = sc[0], pc = cc[0];
    for (int k = 1; k < 7; ++k) {
        ps = ps * x2 + sc[k];
        pc = pc * x2 + cc[k];
    }
    float sn = ps * x;
    switch (q & 3) {
        case 0: s = sn; c = pc; break;
        case 1: s = pc; c = -sn; break;
        case 2: s = -sn; c = -pc; break;
        default: s = -pc; c = sn; break;
    }
}

inline v3 vsub(v3 a, v3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline float vdot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

inline v3 facing_normal(const scene &sc, uint32_t tri, v3 d, uint32_t &mat) {
    const uint32_t *t = sc.t4 + 4 * (size_t)tri;
    mat = t[3];
    v3 a = sc.vert(t[0]), b = sc.vert(t[1]), c = sc.vert(t[2]);
    v3 e1 = vsub(b, a), e2 = vsub(c, a);
    v3 n = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
    float inv = 1.0f / std::sqrt(vdot(n, n));
    n = {n.x * inv, n.y * inv, n.z * inv};
    if (vdot(d, n) > 0.f) n = {-n.x, -n.y, -n.z};
    return n;
}

inline v3 offset_point(v3 o, v3 d, float t, v3 n, float eps) {
    return {(o.x + t * d.x) + eps * n.x, (o.y + t * d.y) + eps * n.y, (o.z + t * d.z) + eps * n.z};
}

inline v3 cosine_dir(float u0, float u1, v3 n) {
    float r = std::sqrt(u0), sn, cs;
    turn_sincos(u1, sn, cs);
    float dx = r * cs, dy = r * sn;
    float z = (1.0f - dx * dx) - dy * dy;
    v3 v = {dx, dy, z > 0.f ? std::sqrt(z) : 0.f};
    float s = std::signbit(n.z) ? -1.0f : 1.0f;
    v3 w = {v.x, v.y, v.z * s};
    v3 hh = {n.x, n.y, n.z + s};
    float k = vdot(w, hh) / (1.0f + (n.z < 0.f ? -n.z : n.z));
    return {k * hh.x - w.x, k * hh.y - w.y, k * hh.z - w.z};
}

inline uint32_t fnv(uint32_t h, uint32_t w) { return (h ^ w) * 16777619u; }
inline uint32_t fbits(float f) {
    uint32_t u;
    std::memcpy(&u, &f, 4);
    return u;
}

struct pt_params {
    uint32_t max_bounces, rr_start;
    float rr_continue, eps;
    uint64_t seed;
};

}  // namespace orc

using namespace orc;

extern "C" {

// Builds the reference BVH over a copy of the scene. split: 0 om, 1 sm, 2 sah.
void *orc_build(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt, int esc, int split, int max_tris,
                int planes) {
    bvh *h = new bvh();
    h->v4.assign(vpos4, vpos4 + 4 * (size_t)nv);
    h->t4.assign(tris4, tris4 + 4 * (size_t)nt);
    h->sc = {h->v4.data(), h->t4.data(), nv, nt};
    builder b(h->sc, split, max_tris, planes, esc != 0);
    h->root = b.build();
    h->nodes.swap(b.nodes);
    h->index.swap(b.index);
    h->failed = b.failed;
    return h;
}

// Texture data for the alpha-aware tracing of orc_closest / orc_any (tc2: 2 floats per vertex;
// mat_tex: texture per material or -1; tex_wh: width and height per texture; texels: the
// textures' alpha values one after another). n_tex = 0 and mat_tex = NULL switch alpha off.
void orc_set_alpha(void *hp, const float *tc2, uint32_t nv, const int32_t *mat_tex, uint32_t n_mat,
                   const uint32_t *tex_wh, const float *texels, uint32_t n_tex) {
    alpha_set &A = ((bvh *)hp)->alpha;
    A = alpha_set();
    if (!mat_tex) return;
    A.on = true;
    A.tc.assign(tc2, tc2 + 2 * (size_t)nv);
    A.mat_tex.assign(mat_tex, mat_tex + n_mat);
    size_t total = 0;
    for (uint32_t k = 0; k < n_tex; ++k) {
        A.w.push_back(tex_wh[2 * k]);
        A.h.push_back(tex_wh[2 * k + 1]);
        A.off.push_back((uint32_t)total);
        total += (size_t)tex_wh[2 * k] * tex_wh[2 * k + 1];
    }
    A.texels.assign(texels, texels + total);
}

int orc_failed(void *hp) { return ((bvh *)hp)->failed ? 1 : 0; }
uint32_t orc_root(void *hp) { return ((bvh *)hp)->root; }
uint32_t orc_num_nodes(void *hp) { return (uint32_t)((bvh *)hp)->nodes.size(); }
uint32_t orc_num_index(void *hp) { return (uint32_t)((bvh *)hp)->index.size(); }

// Same 14-word node layout as the reference harness: l.lo, l.hi, r.lo, r.hi, link_l, link_r.
void orc_get_nodes(void *hp, uint32_t *out) {
    const auto &nodes = ((bvh *)hp)->nodes;
    for (size_t i = 0; i < nodes.size(); ++i) {
        const node &n = nodes[i];
        float f[12] = {n.l.lo.x, n.l.lo.y, n.l.lo.z, n.l.hi.x, n.l.hi.y, n.l.hi.z,
                       n.r.lo.x, n.r.lo.y, n.r.lo.z, n.r.hi.x, n.r.hi.y, n.r.hi.z};
        std::memcpy(out + 14 * i, f, sizeof(f));
        std::memcpy(out + 14 * i + 12, &n.link_l, 4);
        std::memcpy(out + 14 * i + 13, &n.link_r, 4);
    }
}

void orc_get_index(void *hp, uint32_t *out) {
    const auto &idx = ((bvh *)hp)->index;
    std::memcpy(out, idx.data(), idx.size() * 4);
}

// Depth of the tree in edges from the root to the deepest leaf.
uint32_t orc_depth(void *hp) {
    bvh *h = (bvh *)hp;
    std::vector<std::pair<uint32_t, uint32_t>> st = {{h->root, 0}};
    uint32_t best = 0;
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        best = std::max(best, d);
        if (h->nodes[n].inner()) {
            st.push_back({(uint32_t)h->nodes[n].link_l, d + 1});
            st.push_back({(uint32_t)h->nodes[n].link_r, d + 1});
        }
    }
    return best;
}

// Closest hits for a batch (rt/cpu/wavefront.cpp:53-59): out4 = (t, beta, gamma, ref) per ray;
// a miss is t = FLT_MAX, ref = 0 (beta, gamma written as 0). `counts` (optional) receives
// (inner nodes visited, triangle tests, deepest stack index) per ray.
void orc_closest(void *hp, const float *rays8, uint64_t n, float *out4, uint32_t *counts, int threads) {
    bvh *h = (bvh *)hp;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        counters c;
        hit r = closest_hit(*h, load_ray(rays8 + 8 * i), counts ? &c : nullptr);
        float *o = out4 + 4 * i;
        o[0] = r.t;
        o[1] = r.t != FLT_MAX ? r.beta : 0.f;
        o[2] = r.t != FLT_MAX ? r.gamma : 0.f;
        std::memcpy(o + 3, &r.ref, 4);
        if (counts) {
            counts[3 * i] = c.inner;
            counts[3 * i + 1] = c.tris;
            counts[3 * i + 2] = c.max_sp;
        }
    }
}

// Any-hit occlusion flags (rt/cpu/wavefront.cpp:60-70 reduced to the boolean).
void orc_any(void *hp, const float *rays8, uint64_t n, uint8_t *occluded, uint32_t *counts, int threads) {
    bvh *h = (bvh *)hp;
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        counters c;
        occluded[i] = any_hit(*h, load_ray(rays8 + 8 * i), counts ? &c : nullptr) ? 1 : 0;
        if (counts) {
            counts[3 * i] = c.inner;
            counts[3 * i + 1] = c.tris;
            counts[3 * i + 2] = c.max_sp;
        }
    }
}


// Valid hits (t != FLT_MAX) in ray order.
static std::vector<uint32_t> valid_hits(const float *hits4, uint64_t n) {
    std::vector<uint32_t> out;
    for (uint64_t i = 0; i < n; ++i)
        if (hits4[4 * i] != FLT_MAX) out.push_back((uint32_t)i);
    return out;
}

// Shadow rays towards `light`, one per valid hit, in ray order; returns their number.
uint32_t orc_shadow_rays(void *hp, const float *rays8, const float *hits4, uint64_t n, const float *light, float eps,
                         float *out8) {
    bvh *h = (bvh *)hp;
    std::vector<uint32_t> idx = valid_hits(hits4, n);
    for (size_t k = 0; k < idx.size(); ++k) {
        const float *r = rays8 + 8 * (size_t)idx[k];
        const float *hit = hits4 + 4 * (size_t)idx[k];
        uint32_t ref, mat;
        std::memcpy(&ref, hit + 3, 4);
        v3 o = {r[0], r[1], r[2]}, d = {r[4], r[5], r[6]};
        v3 nrm = facing_normal(h->sc, ref, d, mat);
        v3 p = offset_point(o, d, hit[0], nrm, eps);
        v3 to = {light[0] - p.x, light[1] - p.y, light[2] - p.z};
        float dist = std::sqrt(vdot(to, to));
        float *w = out8 + 8 * k;
        w[0] = p.x; w[1] = p.y; w[2] = p.z; w[3] = eps;
        w[4] = to.x / dist; w[5] = to.y / dist; w[6] = to.z / dist; w[7] = dist - eps;
    }
    return (uint32_t)idx.size();
}

// Diffuse paths (see grt_pathtrace): results4 = (radiance, bounces, last_ref, digest) per
// path; bounce_hits (optional) = max_bounces hit records per path, unused slots zero.
void orc_pathtrace(void *hp, const float *prim_rays8, const float *prim_hits4, uint64_t n_primary, uint64_t n_paths,
                   uint32_t max_bounces, uint32_t rr_start, float rr_continue, float eps, uint64_t seed,
                   const float *albedo, uint32_t n_albedo, uint32_t *results4, float *bounce_hits,
                   uint64_t *totals3, int threads) {
    bvh *h = (bvh *)hp;
    set_threads(threads);
    std::vector<uint32_t> H = valid_hits(prim_hits4, n_primary);
    uint64_t t_rays = 0, t_inner = 0, t_tri = 0;
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : t_rays, t_inner, t_tri)
    for (int64_t p = 0; p < (int64_t)n_paths; ++p) {
        uint32_t *res = results4 + 4 * p;
        float *bh = bounce_hits ? bounce_hits + 4 * (size_t)p * max_bounces : nullptr;
        if (bh) std::memset(bh, 0, 16 * (size_t)max_bounces);
        if (H.empty()) {
            float zero = 0.f;
            std::memcpy(res, &zero, 4);
            res[1] = 0;
            res[2] = 0xFFFFFFFFu;
            res[3] = 2166136261u;
            continue;
        }
        uint32_t i = H[(uint64_t)p % H.size()];
        const float *pr = prim_rays8 + 8 * (size_t)i;
        const float *ph = prim_hits4 + 4 * (size_t)i;
        uint32_t pref, mat;
        std::memcpy(&pref, ph + 3, 4);
        v3 o = {pr[0], pr[1], pr[2]}, d = {pr[4], pr[5], pr[6]};
        rng32 rng;
        rng.seq(seed + (uint64_t)p);
        v3 n = facing_normal(h->sc, pref, d, mat);
        v3 org = offset_point(o, d, ph[0], n, eps);
        float u0 = rng.uniform(), u1 = rng.uniform();
        v3 dir = cosine_dir(u0, u1, n);
        float thr = 1.0f, radiance = 0.f;
        uint32_t digest = 2166136261u, last = 0xFFFFFFFFu, bounce = 1;
        for (;;) {
            float rr[8] = {org.x, org.y, org.z, eps, dir.x, dir.y, dir.z, FLT_MAX};
            counters cnt;
            hit hh = closest_hit(*h, load_ray(rr), &cnt);
            t_rays += 1;
            t_inner += cnt.inner;
            t_tri += cnt.tris;
            if (bh) {
                float *w = bh + 4 * (bounce - 1);
                w[0] = hh.t;
                w[1] = hh.t != FLT_MAX ? hh.beta : 0.f;
                w[2] = hh.t != FLT_MAX ? hh.gamma : 0.f;
                std::memcpy(w + 3, &hh.ref, 4);
            }
            if (hh.t == FLT_MAX) {
                digest = fnv(digest, 0xFFFFFFFFu);
                radiance = thr * (0.5f + 0.5f * dir.y);
                break;
            }
            digest = fnv(fnv(digest, hh.ref), fbits(hh.t));
            last = hh.ref;
            v3 nn = facing_normal(h->sc, hh.ref, dir, mat);
            thr = thr * (mat < n_albedo ? albedo[mat] : 0.8f);
            if (bounce >= max_bounces) break;
            if (bounce + 1 >= rr_start) {
                if (!(rng.uniform() < rr_continue)) break;
                thr = thr / rr_continue;
            }
            org = offset_point(org, dir, hh.t, nn, eps);
            u0 = rng.uniform();
            u1 = rng.uniform();
            dir = cosine_dir(u0, u1, nn);
            ++bounce;
        }
        std::memcpy(res, &radiance, 4);
        res[1] = bounce;
        res[2] = last;
        res[3] = digest;
    }
    if (totals3) {
        totals3[0] = t_rays;
        totals3[1] = t_inner;
        totals3[2] = t_tri;
    }
}

// ---- direct lighting ----------------------------------------------------------------------
//
// The reference's CUDA direct-wf steps: k::sample_light with k::sample_index and k::sample_Li
// (rt/cuda/bounce.cu:148-250), the any-hit shadow ray, and k::integrate_light with layered_gtr2
// (bounce.cu:291-339, 380-410; fresnel_dielectric libgi/util.h:91-106, tan2_theta
// libgi/util.h:141-160), over the light distribution of compute_light_distribution
// (rt/cuda/preprocessing.cpp:17-35: luma(trianglelight::power()), libgi/scene.cpp:518-527;
// distribution_1d::build_cdf, libgi/discrete_distributions.cpp:33-45). Geometric normals (the
// shading normal facing the camera ray, a light's normal by its winding), normalize as
// v * (1 / sqrt(v . v)), and the three random numbers of sample s of pixel i from the PCG32
// stream seed + s * n + i. The direction strategies instead draw two numbers from that stream,
// sample uniform_sample_hemisphere (libgi/sampling.h:20-26; pdf one_over_2pi) or
// cosine_sample_hemisphere (pdf one_over_pi * cdot(w_i, n)) around the normal facing the camera
// ray (k::sample_uniform_dir / k::sample_cos_dir, rt/cuda/bounce.cu:33-142), trace a closest-hit
// ray from the hit point (t_min 1e-4) and weight the emission of the triangle it hits
// (k::integrate_dir, bounce.cu:341-375).

struct dl_mat {
    float albedo[3], emissive[3], ior, roughness;
};

struct dl_set {
    std::vector<dl_mat> mats;
    std::vector<uint32_t> lights;  // 4 per light: a, b, c, material
    std::vector<float> f, cdf;
    float integral = 0.f;
    const dl_mat &mat(uint32_t id) const {
        static const dl_mat def = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}, 1.3f, 0.1f};  // libgi/material.h:144-151
        return id < mats.size() ? mats[id] : def;
    }
};

static bool emits(const dl_mat &m) { return m.emissive[0] != 0.f || m.emissive[1] != 0.f || m.emissive[2] != 0.f; }

static dl_set make_dl_set(const scene &sc, const float *mats8, uint32_t n_mat) {
    dl_set L;
    L.mats.resize(n_mat);
    std::memcpy(L.mats.data(), mats8, (size_t)n_mat * sizeof(dl_mat));
    for (uint32_t i = 0; i < sc.nt; ++i) {
        const uint32_t *t = sc.t4 + 4 * (size_t)i;
        if (t[3] >= n_mat || !emits(L.mats[t[3]])) continue;
        const v3 a = sc.vert(t[0]), b = sc.vert(t[1]), c = sc.vert(t[2]);
        const v3 e1 = vsub(b, a), e2 = vsub(c, a);
        const v3 x = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
        const float len = std::sqrt(x.x * x.x + x.y * x.y + x.z * x.z);
        const float pi = 3.14159265358979323846f;
        const float *em = L.mats[t[3]].emissive;
        const float p0 = em[0] * 0.5f * len * pi, p1 = em[1] * 0.5f * len * pi, p2 = em[2] * 0.5f * len * pi;
        L.f.push_back(0.212671f * p0 + 0.715160f * p1 + 0.072169f * p2);
        L.lights.insert(L.lights.end(), {t[0], t[1], t[2], t[3]});
    }
    const size_t N = L.f.size();
    L.cdf.assign(N + 1, 0.f);
    for (size_t i = 1; i <= N; ++i) L.cdf[i] = L.cdf[i - 1] + L.f[i - 1];
    L.integral = L.cdf[N];
    for (size_t i = 1; i <= N; ++i) L.cdf[i] = L.integral > 0.f ? L.cdf[i] / L.integral : (float)i / (float)N;
    return L;
}

static float dl_fresnel(float cos_wi, float ior_medium, float ior_material) {
    const float ei = cos_wi < 0.0f ? ior_material : ior_medium;
    const float et = cos_wi < 0.0f ? ior_medium : ior_material;
    cos_wi = std::fabs(cos_wi);
    cos_wi = cos_wi < 0.0f ? 0.0f : (cos_wi > 1.0f ? 1.0f : cos_wi);
    const float sin_t = (ei / et) * std::sqrt(1.0f - cos_wi * cos_wi);
    if (sin_t >= 1.0f) return 1.0f;
    const float rev = 1.f - sin_t * sin_t;
    const float cos_t = std::sqrt(rev > 0.0f ? rev : 0.0f);
    const float rparl = ((et * cos_wi) - (ei * cos_t)) / ((et * cos_wi) + (ei * cos_t));
    const float rperp = ((ei * cos_wi) - (et * cos_t)) / ((ei * cos_wi) + (et * cos_t));
    return (rparl * rparl + rperp * rperp) / 2;
}

static float dl_tan2(float c) {
    float s2 = 1.0f - c * c;
    s2 = s2 < 0.0f ? 0.0f : s2;
    return s2 / (c * c);
}

static float dl_ggx_d(float nh, float rough) {
    if (nh <= 0) return 0.f;
    const float t2 = dl_tan2(nh);
    if (!std::isfinite(t2)) return 0.f;
    const float a2 = rough * rough;
    const float pi = 3.14159265358979323846f;
    return a2 / (pi * ((nh * nh) * (nh * nh)) * ((a2 + t2) * (a2 + t2)));
}

static float dl_ggx_g1(float nv, float rough) {
    if (nv <= 0) return 0.f;
    const float t2 = dl_tan2(nv);
    if (!std::isfinite(t2)) return 0.f;
    return 2.f / (1.f + std::sqrt(1.f + (rough * rough) * t2));
}

static float cdot3(v3 a, v3 b) {
    const float x = vdot(a, b);
    return x < 0.0f ? 0.0f : x;
}

// layered_gtr2: (1 - F) lambert + F coat
static v3 dl_brdf(v3 w_o, v3 w_i, v3 ns, const dl_mat &m) {
    const float dwo = vdot(ns, w_o);
    const float F = dl_fresnel(dwo < 0.0f ? -dwo : dwo, 1.0f, m.ior);
    const float one_over_pi = (float)(1.0 / 3.14159265358979323846);
    v3 diff = {0.f, 0.f, 0.f};
    if (vdot(w_i, ns) > 0) diff = {one_over_pi * m.albedo[0], one_over_pi * m.albedo[1], one_over_pi * m.albedo[2]};
    float spec = 0.f;
    if (vdot(ns, w_i) > 0) {
        const float nv = cdot3(ns, w_o), nl = cdot3(ns, w_i);
        if (nv != 0.f) {
            v3 h = {w_o.x + w_i.x, w_o.y + w_i.y, w_o.z + w_i.z};
            const float inv = 1.0f / std::sqrt(vdot(h, h));
            h = {h.x * inv, h.y * inv, h.z * inv};
            const float nh = cdot3(ns, h), hl = cdot3(h, w_i);
            const float Fh = dl_fresnel(hl, 1.f, m.ior);
            const float D = dl_ggx_d(nh, m.roughness);
            const float G = dl_ggx_g1(nv, m.roughness) * dl_ggx_g1(nl, m.roughness);
            spec = (Fh * D * G) / (4 * std::fabs(nv) * std::fabs(nl));
        }
    }
    const float k = 1.0f - F;
    return {k * diff.x + F * spec, k * diff.y + F * spec, k * diff.z + F * spec};
}

// a tangent-space sample rotated to the frame of n (align, libgi/util.h:212-218)
static v3 align_to(v3 v, v3 n) {
    const float s = std::signbit(n.z) ? -1.0f : 1.0f;
    const v3 w = {v.x, v.y, v.z * s};
    const v3 hh = {n.x, n.y, n.z + s};
    const float k = vdot(w, hh) / (1.0f + (n.z < 0.f ? -n.z : n.z));
    return {k * hh.x - w.x, k * hh.y - w.y, k * hh.z - w.z};
}

// one pixel: closest hit, then `samples` samples (sampling 0: light, 1: uniform direction,
// 2: cosine-weighted direction) accumulated into fb (4 floats)
static void dl_pixel(const bvh &h, const dl_set &L, const float *ray8, uint32_t pixel, uint32_t n, uint32_t samples,
                     uint64_t seed, uint32_t sampling, float *fb) {
    const ray r = load_ray(ray8);
    const hit ph = closest_hit(h, r, nullptr);
    const v3 o = {ray8[0], ray8[1], ray8[2]}, d = {ray8[4], ray8[5], ray8[6]};
    for (uint32_t s = 0; s < samples; ++s) {
        v3 rad = {0.f, 0.f, 0.f};
        if (ph.t != FLT_MAX) {
            const uint32_t *t = h.sc.t4 + 4 * (size_t)ph.ref;
            const dl_mat &m = L.mat(t[3]);
            if (emits(m)) {
                fb[0] += m.emissive[0];
                fb[1] += m.emissive[1];
                fb[2] += m.emissive[2];
                fb[3] += 0.0f;
            } else if (sampling != 0) {
                rng32 g;
                g.seq(seed + (uint64_t)s * n + pixel);
                const float x0 = g.uniform(), x1 = g.uniform();
                uint32_t mat_id;
                const v3 ns = facing_normal(h.sc, ph.ref, d, mat_id);
                const v3 from = {o.x + ph.t * d.x, o.y + ph.t * d.y, o.z + ph.t * d.z};
                v3 wi;
                float pdf;
                if (sampling == 2) {
                    wi = cosine_dir(x0, x1, ns);
                    pdf = (float)(1.0 / 3.14159265358979323846) * cdot3(wi, ns);
                } else {
                    const float r0 = 1.0f - x0 * x0;
                    const float rr = std::sqrt(r0 < 0.0f ? -r0 : r0);
                    float sn, cs;
                    turn_sincos(x1, sn, cs);
                    wi = align_to({rr * cs, rr * sn, x0}, ns);
                    pdf = (float)(1.0 / (2.0 * 3.14159265358979323846));
                }
                float sr[8] = {from.x, from.y, from.z, 1e-4f, wi.x, wi.y, wi.z, FLT_MAX};
                const hit lh = closest_hit(h, load_ray(sr), nullptr);
                if (lh.t != FLT_MAX) {
                    const float *em = L.mat(h.sc.t4[4 * (size_t)lh.ref + 3]).emissive;
                    const v3 f = dl_brdf({-d.x, -d.y, -d.z}, wi, ns, m);
                    const float cos_t = cdot3(wi, ns);
                    rad = {em[0] * f.x * cos_t / pdf, em[1] * f.y * cos_t / pdf, em[2] * f.z * cos_t / pdf};
                }
            } else if (!L.f.empty()) {
                rng32 g;
                g.seq(seed + (uint64_t)s * n + pixel);
                const float x0 = g.uniform(), x1 = g.uniform(), x2 = g.uniform();
                // sample_index: lower_bound over the first N cdf entries
                int count = (int)L.f.size(), first = 0, i = 0;
                while (count > 0) {
                    i = first;
                    const int step = count / 2;
                    i += step;
                    if (L.cdf[i] < x2) {
                        first = ++i;
                        count -= step + 1;
                    } else {
                        count = step;
                    }
                }
                const int id = i > 0 ? i - 1 : i;
                const float pdf_l = L.f[id] / L.integral;
                const uint32_t *lt = L.lights.data() + 4 * (size_t)id;
                const v3 a = h.sc.vert(lt[0]), b = h.sc.vert(lt[1]), c = h.sc.vert(lt[2]);
                const float *em = L.mat(lt[3]).emissive;
                // sample_Li
                const v3 from = {o.x + ph.t * d.x, o.y + ph.t * d.y, o.z + ph.t * d.z};
                const float su0 = std::sqrt(x0);
                const float bb = 1.0f - su0, bg = x1 * su0;
                const float w = 1.0f - bb - bg;
                const v3 target = {w * a.x + bb * b.x + bg * c.x, w * a.y + bb * b.y + bg * c.y,
                                   w * a.z + bb * b.z + bg * c.z};
                const v3 e1 = vsub(b, a), e2 = vsub(c, a);
                const v3 x = {e1.y * e2.z - e1.z * e2.y, e1.z * e2.x - e1.x * e2.z, e1.x * e2.y - e1.y * e2.x};
                const float inv = 1.0f / std::sqrt(vdot(x, x));
                const v3 ln = {x.x * inv, x.y * inv, x.z * inv};
                v3 wi = vsub(target, from);
                const float area = 0.5f * std::sqrt(vdot(x, x));
                float tmax = std::sqrt(vdot(wi, wi));
                wi = {wi.x / tmax, wi.y / tmax, wi.z / tmax};
                tmax -= 1e-4f;
                const float cos_l = vdot(ln, {-wi.x, -wi.y, -wi.z});
                v3 lcol = {0.f, 0.f, 0.f};
                float a_pdf = 0.f;
                if (cos_l > 0.0f) {
                    lcol = {em[0], em[1], em[2]};
                    a_pdf = tmax * tmax / (cos_l * area);
                }
                const float pdf = pdf_l * a_pdf;
                if ((lcol.x != 0.f || lcol.y != 0.f || lcol.z != 0.f) && tmax > 0.f) {
                    float sr[8] = {from.x, from.y, from.z, 1e-4f, wi.x, wi.y, wi.z, tmax};
                    if (!any_hit(h, load_ray(sr), nullptr)) {
                        uint32_t mat_id;
                        const v3 ns = facing_normal(h.sc, ph.ref, d, mat_id);
                        const v3 f = dl_brdf({-d.x, -d.y, -d.z}, wi, ns, m);
                        const float cos_t = cdot3(wi, ns);
                        rad = {lcol.x * f.x * cos_t / pdf, lcol.y * f.y * cos_t / pdf, lcol.z * f.z * cos_t / pdf};
                    }
                }
            }
        }
        fb[0] += rad.x;
        fb[1] += rad.y;
        fb[2] += rad.z;
        fb[3] += 1.0f;
    }
}

// Direct lighting of n camera rays (8 floats each) into fb (4 floats per ray, accumulated);
// mats8: 8 floats per material (albedo rgb, emission rgb, ior, roughness).
void orc_direct(void *hp, const float *rays8, uint64_t n, const float *mats8, uint32_t n_mat, uint32_t samples,
                uint64_t seed, uint32_t sampling, float *fb, int threads) {
    bvh *h = (bvh *)hp;
    const dl_set L = make_dl_set(h->sc, mats8, n_mat);
    set_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i)
        dl_pixel(*h, L, rays8 + 8 * i, (uint32_t)i, (uint32_t)n, samples, seed, sampling, fb + 4 * i);
}

int orc_max_threads() { return omp_get_max_threads(); }

void orc_free(void *hp) { delete (bvh *)hp; }

}  // extern "C"

// ---- FP64 references for the adjoint (no counterpart in the reference) ---------------------
//
// The intersection of ray (o, d) with a FIXED triangle (A, B, C), in double precision, from the
// same Cramer system as libgi/intersect.h:36-58: beta (A - B) + gamma (A - C) + t d = A - o.
// No range tests: the triangle is given, so the values are defined even outside it.
static void fixed_hit64(const double *A, const double *B, const double *C, const double *o, const double *d,
                        double &t, double &beta, double &gamma) {
    double a = A[0] - B[0], b = A[1] - B[1], c = A[2] - B[2];
    double dd = A[0] - C[0], e = A[1] - C[1], f = A[2] - C[2];
    double g = d[0], h = d[1], i = d[2];
    double j = A[0] - o[0], k = A[1] - o[1], l = A[2] - o[2];
    double c1 = e * i - h * f, c2 = g * f - dd * i, c3 = dd * h - e * g;
    double M = a * c1 + b * c2 + c * c3;
    beta = (j * c1 + k * c2 + l * c3) / M;
    c1 = a * k - j * b;
    c2 = j * c - a * l;
    c3 = b * l - k * c;
    gamma = (i * c1 + h * c2 + g * c3) / M;
    t = -(f * c1 + e * c2 + dd * c3) / M;
}

extern "C" {

// (t, beta, gamma) in double for each ray against its given triangle `refs[i]`.
// vpos3: double [nv, 3]; rays6: double [n, 6] (o, d); out3: double [n, 3].
void orc_fixed_hits64(const double *vpos3, const uint32_t *tris4, const double *rays6, const uint32_t *refs, uint64_t n,
                      double *out3) {
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < (int64_t)n; ++r) {
        const uint32_t *t = tris4 + 4 * (size_t)refs[r];
        fixed_hit64(vpos3 + 3 * (size_t)t[0], vpos3 + 3 * (size_t)t[1], vpos3 + 3 * (size_t)t[2], rays6 + 6 * r,
                    rays6 + 6 * r + 3, out3[3 * r], out3[3 * r + 1], out3[3 * r + 2]);
    }
}

// Analytic adjoint in double: with M = [A-B | A-C | d], x = (beta, gamma, t), g = dL/dx,
// lambda = M^-T g; dA = lambda (1-beta-gamma), dB = lambda beta, dC = lambda gamma,
// do = -lambda, dd = -lambda t. M^-T g is solved by Gaussian elimination with partial
// pivoting (a different method from the kernel's cross products). grad3 per ray is
// (dL/dt, dL/dbeta, dL/dgamma); rays with refs[i] == 0xFFFFFFFF are skipped.
// Outputs: gv3 double [nv, 3] (accumulated), gr6 double [n, 6].
void orc_adjoint64(const double *vpos3, const uint32_t *tris4, const double *rays6, const uint32_t *refs,
                   const double *grad3, uint64_t n, double *gv3, double *gr6) {
    for (uint64_t r = 0; r < n; ++r) {
        double *gr = gr6 + 6 * r;
        for (int q = 0; q < 6; ++q) gr[q] = 0;
        if (refs[r] == 0xFFFFFFFFu) continue;
        const uint32_t *t = tris4 + 4 * (size_t)refs[r];
        const double *A = vpos3 + 3 * (size_t)t[0], *B = vpos3 + 3 * (size_t)t[1], *C = vpos3 + 3 * (size_t)t[2];
        const double *o = rays6 + 6 * r, *d = rays6 + 6 * r + 3;
        double tt, beta, gamma;
        fixed_hit64(A, B, C, o, d, tt, beta, gamma);
        // M^T lambda = g with rows of M^T: (A-B), (A-C), d and g = (g_beta, g_gamma, g_t)
        double m[3][4] = {{A[0] - B[0], A[1] - B[1], A[2] - B[2], grad3[3 * r + 1]},
                          {A[0] - C[0], A[1] - C[1], A[2] - C[2], grad3[3 * r + 2]},
                          {d[0], d[1], d[2], grad3[3 * r + 0]}};
        for (int col = 0; col < 3; ++col) {
            int piv = col;
            for (int row = col + 1; row < 3; ++row)
                if (std::fabs(m[row][col]) > std::fabs(m[piv][col])) piv = row;
            for (int q = 0; q < 4; ++q) std::swap(m[col][q], m[piv][q]);
            for (int row = 0; row < 3; ++row) {
                if (row == col) continue;
                double fct = m[row][col] / m[col][col];
                for (int q = col; q < 4; ++q) m[row][q] -= fct * m[col][q];
            }
        }
        double lam[3] = {m[0][3] / m[0][0], m[1][3] / m[1][1], m[2][3] / m[2][2]};
        for (int q = 0; q < 3; ++q) {
            gv3[3 * (size_t)t[0] + q] += lam[q] * (1.0 - beta - gamma);
            gv3[3 * (size_t)t[1] + q] += lam[q] * beta;
            gv3[3 * (size_t)t[2] + q] += lam[q] * gamma;
            gr[q] = -lam[q];
            gr[3 + q] = -lam[q] * tt;
        }
    }
}

}  // extern "C"
