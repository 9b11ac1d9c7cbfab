// Host-side services around the reference tree of a built scene:
//   * an on-disk cache of reference trees keyed by a hash of the scene and the builder options,
//     so that a scene built once is not built again in a later run (the reference rebuilds on
//     every start; its tracer can only export a tree's boxes, rt/cpu/bvh2.cpp:228-285);
//   * that export (`bvh export <depth> <file.obj>`, rt/cpu/bvh2.cpp:228-283): the child boxes of
//     the inner nodes down to a depth as OBJ quads, in the reference's order and number format;
//   * the leaf statistics of `bvh statistics` (rt/cpu/bvh2.cpp:286-317).
#include <unistd.h>

#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <string>
#include <vector>

#include "ctx.hpp"

using namespace grt;

namespace {

// 128-bit hash of the builder inputs: two independent word-wise multiply-xorshift lanes over the
// vertex and triangle arrays, the counts and the options.
struct hasher {
    uint64_t a = 0x243f6a8885a308d3ull, b = 0x13198a2e03707344ull;
    void word(uint64_t w) {
        a = (a ^ w) * 0x9e3779b97f4a7c15ull;
        a ^= a >> 29;
        b = (b + w) * 0xbf58476d1ce4e5b9ull;
        b ^= b >> 31;
    }
    void bytes(const void *p, size_t n) {
        const unsigned char *c = (const unsigned char *)p;
        size_t i = 0;
        for (; i + 8 <= n; i += 8) {
            uint64_t w;
            std::memcpy(&w, c + i, 8);
            word(w);
        }
        uint64_t tail = 0;
        std::memcpy(&tail, c + i, n - i);
        word(tail ^ ((uint64_t)(n - i) << 56));
    }
};

constexpr char kMagic[8] = {'G', 'R', 'T', 'B', 'V', 'H', 0, 1};
constexpr uint32_t kFormat = 2;

struct file_header {
    char magic[8];
    uint32_t format, nv, nt, root;
    uint64_t key_a, key_b;
    int32_t split, max_tris, planes, esc;
    uint64_t n_nodes, n_index;
    uint64_t body_a, body_b;  // hash of the node and index arrays that follow
};

hasher body_hash(const ref_tree &t) {
    hasher h;
    h.bytes(t.nodes.data(), t.nodes.size() * sizeof(ref_node));
    h.bytes(t.index.data(), t.index.size() * 4);
    return h;
}

std::string cache_path(const std::string &dir, const hasher &h) {
    char name[64];
    std::snprintf(name, sizeof(name), "grt-%016llx%016llx.bvh", (unsigned long long)h.a, (unsigned long long)h.b);
    return dir + "/" + name;
}

hasher key_of(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt, const build_opts &o) {
    hasher h;
    h.word(kFormat);
    h.word(((uint64_t)nv << 32) | nt);
    h.word(((uint64_t)(uint32_t)o.split << 32) | (uint32_t)o.max_tris);
    h.word(((uint64_t)(uint32_t)o.planes << 32) | (o.esc ? 1u : 0u));
    h.bytes(vpos4, (size_t)nv * 16);
    h.bytes(tris4, (size_t)nt * 16);
    return h;
}

// A cached tree is used only if its arrays hash to the value stored with them and every link
// stays inside its arrays and every index names a triangle, so a damaged or foreign file can
// cost a rebuild but never a wrong tree or a bad access.
bool tree_is_sane(const ref_tree &t, uint32_t nt) {
    const size_t nn = t.nodes.size(), ni = t.index.size();
    if (nn == 0 || t.root >= nn) return false;
    for (const ref_node &n : t.nodes) {
        if (n.inner()) {
            if (n.link_l < 0 || (size_t)n.link_l >= nn || (size_t)n.link_r >= nn) return false;
        } else {
            const int64_t first = -(int64_t)n.link_l, count = -(int64_t)n.link_r;
            if (first < 0 || count < 0 || first + count > (int64_t)ni) return false;
        }
    }
    for (uint32_t i : t.index)
        if (i >= nt) return false;
    return true;
}

bool load_tree(const std::string &path, const hasher &h, uint32_t nv, uint32_t nt, const build_opts &o, ref_tree &out) {
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return false;
    file_header hd;
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, kMagic, 8) == 0 && hd.format == kFormat &&
              hd.key_a == h.a && hd.key_b == h.b && hd.nv == nv && hd.nt == nt && hd.split == o.split &&
              hd.max_tris == o.max_tris && hd.planes == o.planes && hd.esc == (o.esc ? 1 : 0) &&
              hd.n_nodes < (1ull << 32) && hd.n_index < (1ull << 32);
    if (ok) {  // the file holds exactly what the header announces (nothing is allocated for a lie)
        const long want = (long)(sizeof(hd) + hd.n_nodes * sizeof(ref_node) + hd.n_index * 4);
        ok = std::fseek(f, 0, SEEK_END) == 0 && std::ftell(f) == want &&
             std::fseek(f, (long)sizeof(hd), SEEK_SET) == 0;
    }
    if (ok) {
        out.root = hd.root;
        out.nodes.resize(hd.n_nodes);
        out.index.resize(hd.n_index);
        ok = std::fread(out.nodes.data(), sizeof(ref_node), hd.n_nodes, f) == hd.n_nodes &&
             std::fread(out.index.data(), 4, hd.n_index, f) == hd.n_index && std::fgetc(f) == EOF;
        if (ok) {
            const hasher b = body_hash(out);
            ok = b.a == hd.body_a && b.b == hd.body_b;
        }
    }
    std::fclose(f);
    return ok && tree_is_sane(out, nt);
}

void store_tree(const std::string &path, const hasher &h, uint32_t nv, uint32_t nt, const build_opts &o,
                const ref_tree &t) {
    // written under a temporary name and renamed, so readers never see a partial file
    const std::string tmp = path + ".tmp" + std::to_string((long)getpid()) + "-" +
                            std::to_string(std::hash<const void *>()(&t));
    FILE *f = std::fopen(tmp.c_str(), "wb");
    if (!f) return;
    file_header hd{};
    std::memcpy(hd.magic, kMagic, 8);
    hd.format = kFormat;
    hd.nv = nv;
    hd.nt = nt;
    hd.root = t.root;
    hd.key_a = h.a;
    hd.key_b = h.b;
    hd.split = o.split;
    hd.max_tris = o.max_tris;
    hd.planes = o.planes;
    hd.esc = o.esc ? 1 : 0;
    hd.n_nodes = t.nodes.size();
    hd.n_index = t.index.size();
    const hasher body = body_hash(t);
    hd.body_a = body.a;
    hd.body_b = body.b;
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
              std::fwrite(t.nodes.data(), sizeof(ref_node), t.nodes.size(), f) == t.nodes.size() &&
              std::fwrite(t.index.data(), 4, t.index.size(), f) == t.index.size();
    ok = std::fclose(f) == 0 && ok;
    if (!ok || std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

void write_box(std::ofstream &out, const float *lo, const float *hi, uint32_t id, uint32_t depth) {
    uint32_t v[8];
    for (int i = 0; i < 8; ++i) v[i] = id * 8 + i + 1;
    out << "v " << lo[0] << " " << lo[1] << " " << lo[2] << "\n";
    out << "v " << hi[0] << " " << lo[1] << " " << lo[2] << "\n";
    out << "v " << hi[0] << " " << hi[1] << " " << lo[2] << "\n";
    out << "v " << lo[0] << " " << hi[1] << " " << lo[2] << "\n";
    out << "v " << lo[0] << " " << lo[1] << " " << hi[2] << "\n";
    out << "v " << hi[0] << " " << lo[1] << " " << hi[2] << "\n";
    out << "v " << hi[0] << " " << hi[1] << " " << hi[2] << "\n";
    out << "v " << lo[0] << " " << hi[1] << " " << hi[2] << "\n";
    out << "g " << "level" << depth + 1 << "\n";
    out << "f " << v[0] << " " << v[1] << " " << v[2] << " " << v[3] << "\n";
    out << "f " << v[1] << " " << v[5] << " " << v[6] << " " << v[2] << "\n";
    out << "f " << v[0] << " " << v[1] << " " << v[5] << " " << v[4] << "\n";
    out << "f " << v[3] << " " << v[2] << " " << v[6] << " " << v[7] << "\n";
    out << "f " << v[4] << " " << v[7] << " " << v[6] << " " << v[5] << "\n";
    out << "f " << v[4] << " " << v[0] << " " << v[3] << " " << v[7] << "\n";
}

}  // namespace

namespace grt {

// The reference build, through the context's cache when one is set.
bool build_or_load(grt_ctx *c, const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt,
                   const build_opts &bo, ref_tree &tree, std::string &err) {
    if (c->cache_dir.empty()) return build_reference_bvh(vpos4, nv, tris4, nt, bo, tree, err);
    const hasher h = key_of(vpos4, nv, tris4, nt, bo);
    const std::string path = cache_path(c->cache_dir, h);
    if (load_tree(path, h, nv, nt, bo, tree)) {
        ++c->cache_hits;
        return true;
    }
    ++c->cache_misses;
    tree = ref_tree();
    if (!build_reference_bvh(vpos4, nv, tris4, nt, bo, tree, err)) return false;
    store_tree(path, h, nv, nt, bo, tree);
    return true;
}

}  // namespace grt

namespace {

bool write_obj(const ref_tree &t, int max_depth, const char *path) {
    std::ofstream out(path, std::ios::trunc);
    if (!out) return false;
    uint32_t id = 0;
    // depth-first: left box and right box of a node, then its left and right subtrees
    std::function<void(uint32_t, uint32_t)> walk = [&](uint32_t node, uint32_t depth) {
        const ref_node &n = t.nodes[node];
        if (!n.inner() || (int64_t)depth >= (int64_t)max_depth) return;
        write_box(out, n.lmin, n.lmax, id++, depth);
        write_box(out, n.rmin, n.rmax, id++, depth);
        walk((uint32_t)n.link_l, depth + 1);
        walk((uint32_t)n.link_r, depth + 1);
    };
    if (!t.nodes.empty()) walk(t.root, 0);
    out.close();
    return (bool)out;
}

// the reference's loop, quirks included: the maximum is only updated when a leaf is not a new
// minimum, and the median of an even count averages positions n/2 and n/2 + 1
const char *leaf_stats(const ref_tree &t, grt_leaf_stats *s) {
    std::vector<int> leaves;
    uint32_t total = 0, count = 0;
    int mx = 0, mn = INT_MAX;
    for (const ref_node &n : t.nodes) {
        if (n.inner()) continue;
        const int k = -n.link_r;
        leaves.push_back(k);
        if (k < mn)
            mn = k;
        else if (k > mx)
            mx = k;
        ++count;
        total += (uint32_t)k;
    }
    if (count == 0) return "the tree has no leaves";
    std::sort(leaves.begin(), leaves.end());
    int median;
    if (count % 2 == 1) {
        median = leaves[leaves.size() / 2];
    } else {
        if (leaves.size() / 2 + 1 >= leaves.size()) return "two leaves: the reference's median reads past the end";
        median = (int)(0.5 * (leaves[leaves.size() / 2] + leaves[leaves.size() / 2 + 1]));
    }
    s->leaves = count;
    s->min_tris = mn;
    s->max_tris = mx;
    s->avg_tris = total / count;
    s->median_tris = median;
    return nullptr;
}

}  // namespace

extern "C" {

grt_status grt_set_bvh_cache(grt_ctx *c, const char *dir) {
    return guarded(c, [&]() -> grt_status {
        if (!c) return GRT_ERR_INVALID_ARG;
        c->cache_dir = dir ? dir : "";
        while (c->cache_dir.size() > 1 && c->cache_dir.back() == '/') c->cache_dir.pop_back();
        if (!c->cache_dir.empty() && access(c->cache_dir.c_str(), W_OK) != 0) {
            const std::string d = c->cache_dir;
            c->cache_dir.clear();
            return fail(c, GRT_ERR_INVALID_ARG, "BVH cache directory '" + d + "' is not writable");
        }
        return GRT_OK;
    });
}

grt_status grt_bvh_cache_stats(const grt_ctx *c, uint64_t *hits, uint64_t *misses) {
    if (!c) return GRT_ERR_INVALID_ARG;
    if (hits) *hits = c->cache_hits;
    if (misses) *misses = c->cache_misses;
    return GRT_OK;
}

grt_status grt_export_bvh_obj(grt_ctx *c, int max_depth, const char *path) {
    return guarded(c, [&]() -> grt_status {
        if (!c || !path) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "no scene has been built");
        if (c->gpu_tree) return fail(c, GRT_ERR_INVALID_ARG, "a BVH built on the GPU or refitted has no reference tree to export");
        return write_obj(c->tree, max_depth, path) ? GRT_OK : fail(c, GRT_ERR_INVALID_ARG, std::string("cannot write ") + path);
    });
}

grt_status grt_bvh_leaf_stats(grt_ctx *c, grt_leaf_stats *s) {
    return guarded(c, [&]() -> grt_status {
        if (!c || !s) return GRT_ERR_INVALID_ARG;
        if (!c->built) return fail(c, GRT_ERR_NOT_BUILT, "no scene has been built");
        if (c->gpu_tree) return fail(c, GRT_ERR_INVALID_ARG, "a BVH built on the GPU or refitted has no reference tree");
        const char *e = leaf_stats(c->tree, s);
        return e ? fail(c, GRT_ERR_INVALID_ARG, e) : GRT_OK;
    });
}

grt_status grt_host_bvh_export_obj(const grt_host_bvh *h, int max_depth, const char *path) {
    return guarded(nullptr, [&]() -> grt_status {
        if (!h || !path) return GRT_ERR_INVALID_ARG;
        return write_obj(host_tree(h), max_depth, path) ? GRT_OK : GRT_ERR_INVALID_ARG;
    });
}

grt_status grt_host_bvh_leaf_stats(const grt_host_bvh *h, grt_leaf_stats *s) {
    return guarded(nullptr, [&]() -> grt_status {
        if (!h || !s) return GRT_ERR_INVALID_ARG;
        return leaf_stats(host_tree(h), s) ? GRT_ERR_INVALID_ARG : GRT_OK;
    });
}

}  // extern "C"
