// Host BVH builder: the reference's CPU SAH / spatial-median / object-median builder with early
// split clipping (rt/cpu/bvh-ctor.h:96-503), restated so that it produces the reference's tree
// node for node (same splits, same leaf order, same box bits, same preorder numbering), and
// organised for large scenes:
//   * primitive centres are computed once instead of per comparison (same float values);
//   * large subtrees are built concurrently; each right subtree is built into its own node list
//     and spliced after the left one with relocated links, which is the reference's preorder;
//   * early split clipping runs in parallel chunks whose extra fragments are appended in
//     triangle order, as the sequential loop appends them.
// std::sort is used wherever the reference sorts, with the same key, because the order it
// leaves equal keys in is part of the tree. Compile with -ffp-contract=off.
#include "bvh_builder.hpp"

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <exception>
#include <functional>
#include <future>
#include <mutex>
#include <system_error>
#include <thread>

namespace grt {
namespace {

// Box with the reference's grow semantics (libgi/intersect.h:5-16 with glm::min/max:
// min(x, y) = (y < x) ? y : x, max(x, y) = (x < y) ? y : x; the order of growth decides the
// sign of zero bounds, so every loop below grows in the reference's order).
struct aabb3 {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX};
    float hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    void add_point(const float *p) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = (lo[k] < p[k]) ? lo[k] : p[k];
            hi[k] = (p[k] < hi[k]) ? hi[k] : p[k];
        }
    }
    void add_box(const aabb3 &b) {
        for (int k = 0; k < 3; ++k) {
            lo[k] = (lo[k] < b.lo[k]) ? lo[k] : b.lo[k];
            hi[k] = (b.hi[k] < hi[k]) ? hi[k] : b.hi[k];
        }
    }
    float surface() const {  // bvh-ctor.h:387-390
        float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
        return 2 * (ex * ey + ex * ez + ey * ez);
    }
    // largest extent axis with the reference's tie order x, y, z (bvh-ctor.h:397-398, 467-475)
    int major_axis() const {
        float ex = hi[0] - lo[0], ey = hi[1] - lo[1], ez = hi[2] - lo[2];
        float m = (ey < ez) ? ez : ey;
        m = (ex < m) ? m : ex;
        return m == ex ? 0 : (m == ey ? 1 : 2);
    }
};

struct builder {
    const float *v4;
    const uint32_t *t4;
    build_opts o;
    std::vector<aabb3> pbox;     // primitive boxes (triangles or ESC fragments)
    std::vector<uint32_t> ptri;  // primitive -> triangle
    std::vector<float> pcen;     // primitive centres, 3 per primitive
    std::vector<uint32_t> index;
    std::atomic<bool> failed{false};
    int par_levels = 0;
    static const uint32_t kParMin = 16384;

    const float *vert(uint32_t i) const { return v4 + 4 * (size_t)i; }

    void set_centres() {
        pcen.resize(pbox.size() * 3);
        for (size_t i = 0; i < pbox.size(); ++i)
            for (int k = 0; k < 3; ++k) pcen[3 * i + k] = (pbox[i].lo[k] + pbox[i].hi[k]) * 0.5f;
    }

    // ---- early split clipping (bvh-ctor.h:120-226) -------------------------------------
    struct p3 {
        float v[3];
    };

    void clip(const std::vector<p3> &poly, float thres, std::vector<aabb3> &out) const {
        aabb3 b;
        for (const p3 &p : poly) b.add_point(p.v);
        if (b.surface() <= thres) {
            out.push_back(b);
            return;
        }
        const int ax = b.major_axis();
        const float mid = (b.hi[ax] + b.lo[ax]) * 0.5f;
        const int n = (int)poly.size();
        // first and second edges (i-1, i) whose endpoints lie on different sides
        int e1 = -1, e2 = -1;
        bool prev = poly[0].v[ax] < mid;
        for (int i = 0; i < n; ++i) {
            bool cur = poly[i].v[ax] < mid;
            if (cur != prev) (e1 == -1 ? e1 : e2) = i - 1;
            prev = cur;
        }
        if (e2 == -1) e2 = n - 1;
        if (e1 == -1) {  // cannot happen for finite input
            out.push_back(b);
            return;
        }
        auto cut = [&](int a) {
            int nb = a + 1 < n ? a + 1 : 0;
            float s = (mid - poly[a].v[ax]) / (poly[nb].v[ax] - poly[a].v[ax]);
            p3 r;
            for (int k = 0; k < 3; ++k) r.v[k] = poly[a].v[k] + (poly[nb].v[k] - poly[a].v[k]) * s;
            return r;
        };
        const p3 c1 = cut(e1), c2 = cut(e2);
        std::vector<p3> lo_part(poly.begin(), poly.begin() + e1 + 1), hi_part;
        lo_part.push_back(c1);
        hi_part.push_back(c1);
        hi_part.insert(hi_part.end(), poly.begin() + e1 + 1, poly.begin() + e2 + 1);
        hi_part.push_back(c2);
        lo_part.push_back(c2);
        lo_part.insert(lo_part.end(), poly.begin() + e2 + 1, poly.end());
        auto eq = [](const p3 &a, const p3 &b) { return a.v[0] == b.v[0] && a.v[1] == b.v[1] && a.v[2] == b.v[2]; };
        lo_part.erase(std::unique(lo_part.begin(), lo_part.end(), eq), lo_part.end());
        hi_part.erase(std::unique(hi_part.begin(), hi_part.end(), eq), hi_part.end());
        clip(lo_part, thres, out);
        clip(hi_part, thres, out);
    }

    void early_split_clipping(int threads) {
        const uint32_t N = (uint32_t)pbox.size();
        std::vector<float> areas(N);
        for (uint32_t i = 0; i < N; ++i) areas[i] = pbox[i].surface();
        const size_t q = 9 * (size_t)N / 10;
        std::nth_element(areas.begin(), areas.begin() + q, areas.end());
        const float thres = areas[q];
        // each chunk keeps its extra fragments in triangle order; chunks are appended in order
        int chunks = (N >= 65536 && threads > 1) ? threads * 4 : 1;
        std::vector<std::vector<std::pair<aabb3, uint32_t>>> extra(chunks);
        auto work = [&](int c) {
            uint32_t b = (uint32_t)((uint64_t)N * c / chunks), e = (uint32_t)((uint64_t)N * (c + 1) / chunks);
            std::vector<aabb3> gen;
            std::vector<p3> poly(3);
            for (uint32_t i = b; i < e; ++i) {
                if (pbox[i].surface() <= thres) continue;  // clip() would return the box unchanged
                const uint32_t *t = t4 + 4 * (size_t)i;
                for (int k = 0; k < 3; ++k) std::memcpy(poly[k].v, vert(t[k]), 12);
                gen.clear();
                clip(poly, thres, gen);
                pbox[i] = gen[0];
                for (size_t j = 1; j < gen.size(); ++j) extra[c].push_back({gen[j], i});
            }
        };
        if (chunks == 1) {
            work(0);
        } else {
            // the threads that start share the chunks (the calling thread takes them all if none
            // starts); an exception in one, such as memory running out, is raised after the join
            std::vector<std::thread> th;
            std::atomic<int> next{0};
            std::exception_ptr failed;
            std::mutex failed_mutex;
            auto run = [&] {
                try {
                    for (int c; (c = next++) < chunks;) work(c);
                } catch (...) {
                    std::lock_guard<std::mutex> lock(failed_mutex);
                    if (!failed) failed = std::current_exception();
                    next = chunks;
                }
            };
            th.reserve(threads);
            for (int t = 0; t < threads; ++t) {
                try {
                    th.emplace_back(run);
                } catch (const std::system_error &) {
                    break;
                }
            }
            if (th.empty()) run();
            for (auto &t : th) t.join();
            if (failed) std::rethrow_exception(failed);
        }
        for (auto &ex : extra)
            for (auto &pr : ex) {
                pbox.push_back(pr.first);
                ptri.push_back(pr.second);
                index.push_back((uint32_t)pbox.size() - 1);
            }
    }

    // ---- subdivision ---------------------------------------------------------------------
    float cen(uint32_t p, int ax) const { return pcen[3 * (size_t)p + ax]; }

    void sort_by_centre(uint32_t s, uint32_t e, int ax) {
        std::sort(index.begin() + s, index.begin() + e,
                  [&](uint32_t a, uint32_t b) { return cen(a, ax) < cen(b, ax); });
    }

    aabb3 span_box(uint32_t s, uint32_t e) const {
        aabb3 b;
        for (uint32_t i = s; i < e; ++i) b.add_box(pbox[index[i]]);
        return b;
    }

    // In-place two-pointer partition by centre <= plane (bvh-ctor.h:333-343, 427-440),
    // including its quirk of never classifying the element where the pointers meet.
    uint32_t partition(uint32_t s, uint32_t e, int ax, float plane) {
        uint32_t mid = s;
        uint32_t *L = index.data() + s, *R = index.data() + e - 1;
        while (L < R) {
            while (L < R && cen(*L, ax) <= plane) ++L, ++mid;
            while (L < R && cen(*R, ax) > plane) --R;
            if (L < R && cen(*L, ax) > cen(*R, ax)) std::swap(*L, *R);
        }
        return mid;
    }

    static ref_node leaf(uint32_t s, uint32_t e) {
        ref_node n{};
        for (int k = 0; k < 3; ++k) {
            n.lmin[k] = n.rmin[k] = FLT_MAX;
            n.lmax[k] = n.rmax[k] = -FLT_MAX;
        }
        n.link_l = -(int32_t)s;
        n.link_r = -(int32_t)(e - s);
        return n;
    }

    static void put_boxes(ref_node &n, const aabb3 &l, const aabb3 &r) {
        for (int k = 0; k < 3; ++k) {
            n.lmin[k] = l.lo[k];
            n.lmax[k] = l.hi[k];
            n.rmin[k] = r.lo[k];
            n.rmax[k] = r.hi[k];
        }
    }

    // Chooses the split of [s, e); returns false for a leaf. For SAH the child boxes come from
    // the winning candidate (bvh-ctor.h:453-459); OM and SM grow them after the recursion.
    bool choose_split(uint32_t s, uint32_t e, uint32_t &mid, aabb3 &bl, aabb3 &br) {
        const aabb3 b = span_box(s, e);
        const int ax = b.major_axis();
        if (o.split == 0) {  // object median (bvh-ctor.h:266-285)
            sort_by_centre(s, e, ax);
            mid = s + (e - s) / 2;
            return true;
        }
        if (o.split == 1) {  // spatial median (bvh-ctor.h:317-353)
            float plane = b.lo[ax] + (b.hi[ax] - b.lo[ax]) * 0.5f;
            mid = partition(s, e, ax, plane);
            if (mid == s || mid == e - 1) {
                sort_by_centre(s, e, ax);
                mid = s + (e - s) / 2;
            }
            return true;
        }
        // SAH (bvh-ctor.h:386-488)
        const float surf = b.surface();
        mid = s;
        if (surf == 0) {
            sort_by_centre(s, e, ax);
            mid = s + (e - s) / 2;
            bl = span_box(s, mid);
            br = span_box(mid, e);
            return true;
        }
        float best_l = FLT_MAX, best_r = FLT_MAX;
        bool median_left = true;
        int planes = o.planes;
        if ((int)(e - s) < planes) planes = (int)(e - s);
        const float ext = b.hi[ax] - b.lo[ax];
        for (int i = 0; i < planes; ++i) {
            const float plane = b.lo[ax] + (float)(i + 1) * (ext / (float)(planes + 1));
            uint32_t cut = partition(s, e, ax, plane);
            if (cut == s || cut == e - 1) {
                if (!median_left) continue;
                sort_by_centre(s, e, ax);
                cut = s + (e - s) / 2;
                median_left = false;
            }
            aabb3 cl = span_box(s, cut), cr = span_box(cut, e);
            float cost_l = (cl.surface() / surf) * (float)(cut - s);
            float cost_r = (cr.surface() / surf) * (float)(e - cut);
            if (cost_l + cost_r < best_l + best_r) {
                bl = cl;
                br = cr;
                best_l = cost_l;
                best_r = cost_r;
                mid = cut;
            }
        }
        // bvh-ctor.h:479-487 can only make a leaf of at most max_tris primitives, and such
        // ranges never get here, so the SAH termination test is never taken.
        if (mid == s) {
            failed = true;  // no candidate was accepted (non-finite input); the reference recurses forever
            return false;
        }
        return true;
    }

    uint32_t subdivide(uint32_t s, uint32_t e, std::vector<ref_node> &out, int par) {
        if (e - s <= (uint32_t)o.max_tris || failed) {
            out.push_back(leaf(s, e));
            return (uint32_t)out.size() - 1;
        }
        uint32_t mid;
        aabb3 bl, br;
        if (!choose_split(s, e, mid, bl, br)) {
            out.push_back(leaf(s, e));
            return (uint32_t)out.size() - 1;
        }
        const uint32_t id = (uint32_t)out.size();
        out.emplace_back();
        uint32_t l, r;
        if (par > 0 && e - s >= kParMin) {
            std::vector<ref_node> right;
            auto fut = std::async(std::launch::async, [&] { return subdivide(mid, e, right, par - 1); });
            l = subdivide(s, mid, out, par - 1);
            const uint32_t rl = fut.get();
            const int32_t off = (int32_t)out.size();
            for (ref_node n : right) {
                if (n.inner()) {
                    n.link_l += off;
                    n.link_r += off;
                }
                out.push_back(n);
            }
            r = rl + (uint32_t)off;
        } else {
            l = subdivide(s, mid, out, 0);
            r = subdivide(mid, e, out, 0);
        }
        ref_node &n = out[id];
        n.link_l = (int32_t)l;
        n.link_r = (int32_t)r;
        if (o.split == 2)
            put_boxes(n, bl, br);
        else
            put_boxes(n, span_box(s, mid), span_box(mid, e));
        return id;
    }
};

}  // namespace

bool build_reference_bvh(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt, const build_opts &opts,
                         ref_tree &out, std::string &err) {
    if (opts.split < 0 || opts.split > 2 || opts.max_tris < 1 || opts.max_tris > (int)kMaxLeafTris ||
        opts.planes < 1) {
        err = "invalid BVH options";
        return false;
    }
    for (uint32_t t = 0; t < nt; ++t)
        for (int k = 0; k < 3; ++k)
            if (tris4[4 * (size_t)t + k] >= nv) {
                err = "triangle " + std::to_string(t) + " references vertex " +
                      std::to_string(tris4[4 * (size_t)t + k]) + " >= nv";
                return false;
            }
    builder b;
    b.v4 = vpos4;
    b.t4 = tris4;
    b.o = opts;
    int threads = opts.threads > 0 ? opts.threads : (int)std::max(1u, std::thread::hardware_concurrency());
    b.par_levels = 0;
    while ((1 << b.par_levels) < 4 * threads && b.par_levels < 8) ++b.par_levels;
    b.pbox.resize(nt);
    b.ptri.resize(nt);
    b.index.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) {
        const uint32_t *t = tris4 + 4 * (size_t)i;
        aabb3 box;
        for (int k = 0; k < 3; ++k) box.add_point(b.vert(t[k]));
        b.pbox[i] = box;
        b.ptri[i] = i;
        b.index[i] = i;
    }
    // The reference cannot clip an empty scene (it reads the 90th-percentile primitive).
    if (opts.esc && nt > 0) b.early_split_clipping(threads);
    b.set_centres();
    out.nodes.clear();
    out.nodes.reserve(2 * b.pbox.size() / std::max(1, opts.max_tris) + 2);
    out.root = b.subdivide(0, (uint32_t)b.pbox.size(), out.nodes, b.par_levels);
    if (b.failed) {
        err = "the builder found no split of a node (non-finite vertex coordinates?)";
        return false;
    }
    out.index.resize(b.index.size());
    for (size_t i = 0; i < b.index.size(); ++i) out.index[i] = b.ptri[b.index[i]];
    return true;
}

bool flatten_bvh(const ref_tree &tree, const float *vpos4, const uint32_t *tris4, flat_bvh &out, std::string &err) {
    out = flat_bvh();
    if (tree.index.size() >= kMaxRecords) {
        err = "too many triangle records for the device layout";
        return false;
    }
    const auto &N = tree.nodes;
    if (tree.index.empty()) {  // no triangles: the reference's single leaf of count 0
        out.empty = true;
        return true;
    }
    // inner nodes keep the reference preorder, leaves are folded into their parents
    std::vector<int32_t> inner_id(N.size(), -1);
    uint32_t inner = 0;
    for (size_t i = 0; i < N.size(); ++i)
        if (N[i].inner()) inner_id[i] = (int32_t)inner++;
    auto child_ref = [&](int32_t link, bool &ok) -> int32_t {
        const ref_node &c = N[link];
        if (c.inner()) return inner_id[link];
        uint32_t first = (uint32_t)(-c.link_l), count = (uint32_t)(-c.link_r);
        if (count == 0 || count > kMaxLeafTris) ok = false;
        return ~(int32_t)((first << 4) | (count - 1));
    };
    out.inner = inner;
    out.nodes.assign((size_t)inner * 16, 0.f);
    out.parent.assign(inner, -1);
    bool ok = true;
    for (size_t i = 0; i < N.size(); ++i) {
        if (!N[i].inner()) continue;
        const ref_node &n = N[i];
        float *d = out.nodes.data() + (size_t)inner_id[i] * 16;
        int32_t cl = child_ref(n.link_l, ok), cr = child_ref(n.link_r, ok);
        if (cl >= 0) out.parent[cl] = inner_id[i] * 2;
        if (cr >= 0) out.parent[cr] = inner_id[i] * 2 + 1;
        const float *lo[2] = {n.lmin, n.rmin}, *hi[2] = {n.lmax, n.rmax};
        const int32_t ref[2] = {cl, cr};
        for (int side = 0; side < 2; ++side) {
            float *e = d + 8 * side;
            e[0] = lo[side][0];
            e[1] = lo[side][1];
            e[2] = hi[side][0];
            e[3] = hi[side][1];
            e[4] = lo[side][2];
            e[5] = hi[side][2];
            std::memcpy(e + 6, &ref[side], 4);
        }
    }
    out.inner_id = std::move(inner_id);
    const ref_node &root = N[tree.root];
    if (root.inner()) {
        out.root = out.inner_id[tree.root];
    } else if (root.link_r == 0) {
        out.empty = true;
        out.root = 0;
    } else {
        out.root = child_ref((int32_t)tree.root, ok);
    }
    if (!ok) {
        err = "a leaf holds more triangles than the device layout allows";
        return false;
    }
    // depth in edges
    std::vector<std::pair<uint32_t, uint32_t>> st = {{tree.root, 0}};
    while (!st.empty()) {
        auto [n, d] = st.back();
        st.pop_back();
        if (d > out.depth) out.depth = d;
        if (N[n].inner()) {
            st.push_back({(uint32_t)N[n].link_l, d + 1});
            st.push_back({(uint32_t)N[n].link_r, d + 1});
        }
    }
    out.records.resize(tree.index.size() * 12);
    for (size_t i = 0; i < tree.index.size(); ++i) {
        const uint32_t tri = tree.index[i];
        const uint32_t *t = tris4 + 4 * (size_t)tri;
        const float *a = vpos4 + 4 * (size_t)t[0], *b = vpos4 + 4 * (size_t)t[1], *c = vpos4 + 4 * (size_t)t[2];
        float *r = out.records.data() + 12 * i;
        r[0] = a[0];
        r[1] = a[1];
        r[2] = a[2];
        std::memcpy(r + 3, &tri, 4);
        r[4] = a[0] - b[0];
        r[5] = a[1] - b[1];
        r[6] = a[2] - b[2];
        std::memcpy(r + 7, t + 3, 4);  // material id, for shading without a triangle fetch
        r[8] = a[0] - c[0];
        r[9] = a[1] - c[1];
        r[10] = a[2] - c[2];
        r[11] = 0.f;
    }
    return true;
}

bool flatten_bvh4(const ref_tree &tree, const flat_bvh &flat, flat_bvh4 &out, std::string &err) {
    out = flat_bvh4();
    if (flat.empty) return true;
    const auto &N = tree.nodes;
    auto leaf_ref = [&](int32_t link) {
        const ref_node &c = N[link];
        uint32_t first = (uint32_t)(-c.link_l), count = (uint32_t)(-c.link_r);
        return ~(int32_t)((first << 4) | (count - 1));
    };
    if (!N[tree.root].inner()) {
        out.root = leaf_ref((int32_t)tree.root);
        return true;
    }
    struct child {
        float lo[3], hi[3];
        int32_t link;  // reference node
    };
    // explicit stack of (reference inner node, wide slot); wide slots are assigned in preorder
    std::vector<std::pair<uint32_t, uint32_t>> todo;
    std::vector<uint32_t> bound;   // stack bound of the subtree under each wide node
    std::vector<std::vector<uint32_t>> kids;  // wide children of each wide node
    auto new_node = [&]() {
        out.nodes.resize(out.nodes.size() + 32, 0.f);
        kids.emplace_back();
        return (uint32_t)(out.nodes.size() / 32 - 1);
    };
    // recursive lambda via explicit function object (depth is at most the reference depth)
    out.wide_index.assign(flat.inner + 1, -1);  // one entry past the last node, as the GPU builder's
    std::function<uint32_t(uint32_t)> build = [&](uint32_t bin) -> uint32_t {
        const uint32_t w = new_node();
        out.wide_index[flat.inner_id[bin]] = (int32_t)w;
        const ref_node &n = N[bin];
        child ch[4];
        int k = 0;
        const float *boxes[2][2] = {{n.lmin, n.lmax}, {n.rmin, n.rmax}};
        const int32_t links[2] = {n.link_l, n.link_r};
        for (int side = 0; side < 2; ++side) {
            const ref_node &c = N[links[side]];
            if (c.inner()) {
                const float *gb[2][2] = {{c.lmin, c.lmax}, {c.rmin, c.rmax}};
                const int32_t gl[2] = {c.link_l, c.link_r};
                for (int g = 0; g < 2; ++g) {
                    std::memcpy(ch[k].lo, gb[g][0], 12);
                    std::memcpy(ch[k].hi, gb[g][1], 12);
                    ch[k++].link = gl[g];
                }
            } else {
                std::memcpy(ch[k].lo, boxes[side][0], 12);
                std::memcpy(ch[k].hi, boxes[side][1], 12);
                ch[k++].link = links[side];
            }
        }
        int32_t ref[4];
        for (int i = 0; i < 4; ++i) {
            if (i >= k) {
                ref[i] = kEmptyChild;
            } else if (N[ch[i].link].inner()) {
                const uint32_t cw = build((uint32_t)ch[i].link);
                kids[w].push_back(cw);
                ref[i] = (int32_t)cw;
            } else {
                ref[i] = leaf_ref(ch[i].link);
            }
        }
        float *d = out.nodes.data() + 32 * (size_t)w;
        for (int i = 0; i < 4; ++i) {
            const bool used = i < k;
            const float inf = __builtin_inff();
            float *e = d + 8 * i;
            e[0] = used ? ch[i].lo[0] : inf;
            e[1] = used ? ch[i].lo[1] : inf;
            e[2] = used ? ch[i].hi[0] : inf;
            e[3] = used ? ch[i].hi[1] : inf;
            e[4] = used ? ch[i].lo[2] : inf;
            e[5] = used ? ch[i].hi[2] : inf;
            std::memcpy(e + 6, &ref[i], 4);
        }
        uint32_t sub = 0;
        for (uint32_t cw : kids[w]) sub = std::max(sub, bound[cw]);
        if (bound.size() <= w) bound.resize(w + 1, 0);
        bound[w] = (uint32_t)(k - 1) + sub;
        return w;
    };
    bound.reserve(N.size());
    out.root = (int32_t)build(tree.root);
    out.count = (uint32_t)(out.nodes.size() / 32);
    out.stack_bound = bound[0];
    (void)err;
    return true;
}

}  // namespace grt
