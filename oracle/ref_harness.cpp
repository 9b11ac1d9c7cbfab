// Test-infrastructure harness around the reference's own CPU ray tracer.
//
// This file is compiled together with the UNMODIFIED reference sources rt/cpu/bvh2.cpp,
// libgi/timer.cpp and libgi/rt.cpp (by oracle/build_ref.sh, into oracle/_ref/libref_bbvh.so)
// and exposes the reference's binary_bvh_tracer (rt/cpu/bvh.h:68-106) through a few
// extern "C" functions so that the oracle restatement and the golden fixtures can be checked
// against the reference itself. Only the tests and the fixture generator load it. It never
// ships: the reference sources are not in this repository and the library is git-ignored.
//
// Configuration mirrors the CUDA platform's batch tracer build (rt/cuda/base.cpp:88-117):
// indexed triangle layout, SAH with `planes` uniform planes, `max_tris` triangles per leaf and
// early split clipping on or off.
#include "rt/cpu/bvh.h"

#include <cstdint>
#include <cstring>
#include <iostream>
#include <omp.h>
#include <sstream>

// The harness needs no scene teardown beyond the member vectors (libgi/scene.cpp is not built:
// it needs assimp and ImageMagick).
scene::~scene() {}

namespace {

typedef binary_bvh_tracer<bbvh_triangle_layout::indexed, bbvh_esc_mode::on> tracer_esc;
typedef binary_bvh_tracer<bbvh_triangle_layout::indexed, bbvh_esc_mode::off> tracer_noesc;
// the alpha-aware variant the reference instantiates (rt/cpu/bvh2.cpp:324)
typedef binary_bvh_tracer<bbvh_triangle_layout::indexed, bbvh_esc_mode::on, true> tracer_alpha;

struct handle {
    ::scene sc;
    individual_ray_tracer *rt = nullptr;
    ::bvh *bvh = nullptr;
    std::vector<texture2d<vec4> *> owned;  // textures of the alpha-aware scene
};

template <typename T> void configure_and_build(handle *h, int split, int max_tris, int planes) {
    T *t = new T();
    t->binary_split_type = split == 0 ? T::om : (split == 1 ? T::sm : T::sah);
    t->max_triangles_per_node = max_tris;
    t->number_of_planes = planes;
    t->build(&h->sc);
    h->rt = t;
    h->bvh = &t->bvh;
}

ray make_ray(const float *r) {
    // GPU ray layout: (o.xyz, t_min), (d.xyz, t_max); the CPU ray recomputes id = 1/d.
    ray out(vec3(r[0], r[1], r[2]), vec3(r[4], r[5], r[6]));
    out.t_min = r[3];
    out.t_max = r[7];
    return out;
}

}  // namespace

extern "C" {

void *ref_build(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt, int esc, int split,
                int max_tris, int planes) {
    handle *h = new handle();
    h->sc.vertices.resize(nv);
    for (uint32_t i = 0; i < nv; ++i) {
        h->sc.vertices[i].pos = vec3(vpos4[4 * i + 0], vpos4[4 * i + 1], vpos4[4 * i + 2]);
        h->sc.vertices[i].norm = vec3(0, 0, 1);
        h->sc.vertices[i].tc = vec2(0, 0);
    }
    h->sc.triangles.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) {
        h->sc.triangles[i].a = tris4[4 * i + 0];
        h->sc.triangles[i].b = tris4[4 * i + 1];
        h->sc.triangles[i].c = tris4[4 * i + 2];
        h->sc.triangles[i].material_id = tris4[4 * i + 3];
    }
    if (esc)
        configure_and_build<tracer_esc>(h, split, max_tris, planes);
    else
        configure_and_build<tracer_noesc>(h, split, max_tris, planes);
    return h;
}

// The alpha-aware tracer (ESC on, SAH) over a scene with texture coordinates (tc2: 2 per
// vertex), a texture per material (mat_tex, -1 for none; the material table has n_mat entries)
// and alpha textures (tex_wh: width, height per texture; texels: alpha values one texture after
// another, stored as the w channel of the reference's vec4 texels).
void *ref_build_alpha(const float *vpos4, uint32_t nv, const uint32_t *tris4, uint32_t nt, const float *tc2,
                      const int32_t *mat_tex, uint32_t n_mat, const uint32_t *tex_wh, const float *texels,
                      uint32_t n_tex, int max_tris, int planes) {
    handle *h = new handle();
    h->sc.vertices.resize(nv);
    for (uint32_t i = 0; i < nv; ++i) {
        h->sc.vertices[i].pos = vec3(vpos4[4 * i + 0], vpos4[4 * i + 1], vpos4[4 * i + 2]);
        h->sc.vertices[i].norm = vec3(0, 0, 1);
        h->sc.vertices[i].tc = vec2(tc2[2 * i], tc2[2 * i + 1]);
    }
    h->sc.triangles.resize(nt);
    for (uint32_t i = 0; i < nt; ++i) {
        h->sc.triangles[i].a = tris4[4 * i + 0];
        h->sc.triangles[i].b = tris4[4 * i + 1];
        h->sc.triangles[i].c = tris4[4 * i + 2];
        h->sc.triangles[i].material_id = tris4[4 * i + 3];
    }
    size_t off = 0;
    for (uint32_t k = 0; k < n_tex; ++k) {
        texture2d<vec4> *t = new texture2d<vec4>();
        t->w = tex_wh[2 * k];
        t->h = tex_wh[2 * k + 1];
        t->texel = new vec4[(size_t)t->w * t->h];
        for (size_t q = 0; q < (size_t)t->w * t->h; ++q) t->texel[q] = vec4(0, 0, 0, texels[off + q]);
        off += (size_t)t->w * t->h;
        h->owned.push_back(t);
    }
    h->sc.materials.resize(n_mat);
    for (uint32_t m = 0; m < n_mat; ++m)
        h->sc.materials[m].albedo_tex = mat_tex[m] >= 0 ? h->owned[mat_tex[m]] : nullptr;
    configure_and_build<tracer_alpha>(h, 2, max_tris, planes);
    return h;
}

uint32_t ref_root(void *hp) { return ((handle *)hp)->bvh->root; }
uint32_t ref_num_nodes(void *hp) { return (uint32_t)((handle *)hp)->bvh->nodes.size(); }
uint32_t ref_num_index(void *hp) { return (uint32_t)((handle *)hp)->bvh->index.size(); }

// Nodes as 14 x 32-bit words each: box_l.min xyz, box_l.max xyz, box_r.min xyz, box_r.max xyz,
// link_l, link_r (the bbvh_node field order, rt/cpu/bvh.h:42-52).
void ref_get_nodes(void *hp, uint32_t *out) {
    const auto &nodes = ((handle *)hp)->bvh->nodes;
    for (size_t i = 0; i < nodes.size(); ++i) {
        const bbvh_node &n = nodes[i];
        float f[12] = {n.box_l.min.x, n.box_l.min.y, n.box_l.min.z, n.box_l.max.x, n.box_l.max.y, n.box_l.max.z,
                       n.box_r.min.x, n.box_r.min.y, n.box_r.min.z, n.box_r.max.x, n.box_r.max.y, n.box_r.max.z};
        std::memcpy(out + 14 * i, f, sizeof(f));
        std::memcpy(out + 14 * i + 12, &n.link_l, 4);
        std::memcpy(out + 14 * i + 13, &n.link_r, 4);
    }
}

void ref_get_index(void *hp, uint32_t *out) {
    const auto &idx = ((handle *)hp)->bvh->index;
    std::memcpy(out, idx.data(), idx.size() * 4);
}

// Closest hits in the layout of rt/cpu/wavefront.cpp:53-59 (one triangle_intersection per ray),
// written as (t, beta, gamma, ref). A miss leaves beta/gamma as the reference leaves them
// (uninitialised); the harness zeroes them first so the output is deterministic.
void ref_closest(void *hp, const float *rays8, uint32_t n, float *out4, int threads) {
    handle *h = (handle *)hp;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
        triangle_intersection is = h->rt->closest_hit(make_ray(rays8 + 8 * i));
        float *o = out4 + 4 * i;
        o[0] = is.t;
        o[1] = is.valid() ? is.beta : 0.f;
        o[2] = is.valid() ? is.gamma : 0.f;
        std::memcpy(o + 3, &is.ref, 4);
    }
}

// Any-hit flags (1 = occluded), rt/cpu/wavefront.cpp:60-70 reduced to the bool.
void ref_any(void *hp, const float *rays8, uint32_t n, uint8_t *occluded, int threads) {
    handle *h = (handle *)hp;
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < (int64_t)n; ++i) occluded[i] = h->rt->any_hit(make_ray(rays8 + 8 * i)) ? 1 : 0;
}

// Runs the reference tracer's own script command `bvh <args>` (binary_bvh_tracer::interprete,
// rt/cpu/bvh2.cpp:192-241) and returns what it printed on stdout (at most cap - 1 bytes).
int ref_bvh_command(void *hp, const char *args, char *out, int cap) {
    handle *h = (handle *)hp;
    std::ostringstream captured;
    std::streambuf *old = std::cout.rdbuf(captured.rdbuf());
    std::istringstream in(args);
    const bool ok = h->rt->interprete("bvh", in);
    std::cout.rdbuf(old);
    const std::string s = captured.str();
    const int n = (int)std::min<size_t>(s.size(), cap > 0 ? (size_t)cap - 1 : 0);
    if (cap > 0) {
        std::memcpy(out, s.data(), n);
        out[n] = 0;
    }
    return ok ? 1 : 0;
}

void ref_free(void *hp) {
    handle *h = (handle *)hp;
    delete h->rt;
    for (texture2d<vec4> *t : h->owned) delete t;
    delete h;
}

}  // extern "C"
