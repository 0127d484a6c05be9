// Host-side scene construction.
//
// The BVH topology is the reference's: a 12-bucket binned SAH over centroid
// bounds with its cost formula, leaf/recursion rules and node order
// (Core/BVH.cpp:73-107 BVHFactory::split_primitives, Core/BVH.cpp:126-197
// SAH_parition_Scheme::partition), with std::partition doing the reordering as
// the reference does, so leaves hold the same items in the same order.  The
// inputs match too: per-triangle bounds for a BLAS
// (Core/LowerLevelMeshBVH.cpp:48-64), the mesh AABB transformed corner by
// corner for a TLAS entry (Core/UpperLevelBVH.cpp:27-57, Core/AABB.cpp:253-270).
// Float arithmetic follows glm's operation order and this file is compiled
// with -ffp-contract=off, so boxes, inverses and light tables are bit-identical
// to the reference's.
//
// The topology is then flattened into the 64-byte child-box node layout of
// layout.h.  Leaves larger than 31 items (only degenerate inputs make them)
// become chains of nodes that repeat the leaf's box, which keeps the item
// order and therefore the ranks.
#include "scene_build.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <limits>

namespace pico {
namespace {

constexpr uint32_t kInvalid = 0xffffffffu;
constexpr float kInf = std::numeric_limits<float>::infinity();

struct V4 { float x, y, z, w; };

inline float sel_min(float a, float b) { return (b < a) ? b : a; }   // glm::min
inline float sel_max(float a, float b) { return (a < b) ? b : a; }   // glm::max

struct Box {
    V4 lo{kInf, kInf, kInf, kInf};
    V4 hi{-kInf, -kInf, -kInf, -kInf};

    void grow(const Box& o)
    {
        lo = {sel_min(lo.x, o.lo.x), sel_min(lo.y, o.lo.y), sel_min(lo.z, o.lo.z), sel_min(lo.w, o.lo.w)};
        hi = {sel_max(hi.x, o.hi.x), sel_max(hi.y, o.hi.y), sel_max(hi.z, o.hi.z), sel_max(hi.w, o.hi.w)};
    }
    void grow(const V4& p)
    {
        lo = {sel_min(lo.x, p.x), sel_min(lo.y, p.y), sel_min(lo.z, p.z), sel_min(lo.w, p.w)};
        hi = {sel_max(hi.x, p.x), sel_max(hi.y, p.y), sel_max(hi.z, p.z), sel_max(hi.w, p.w)};
    }
    V4 center() const
    {
        return {lo.x + (hi.x - lo.x) * 0.5f, lo.y + (hi.y - lo.y) * 0.5f, lo.z + (hi.z - lo.z) * 0.5f,
                lo.w + (hi.w - lo.w) * 0.5f};
    }
    void sides(float s[3]) const
    {
        s[0] = std::fabs(hi.x - lo.x); s[1] = std::fabs(hi.y - lo.y); s[2] = std::fabs(hi.z - lo.z);
    }
    float area() const
    {
        float s[3];
        sides(s);
        return 2.0f * (((s[0] * s[1]) + (s[0] * s[2])) + (s[1] * s[2]));
    }
    float offset(const V4& p, int axis) const
    {
        float o[3] = {p.x - lo.x, p.y - lo.y, p.z - lo.z};
        if (hi.x > lo.x) o[0] /= hi.x - lo.x;
        if (hi.y > lo.y) o[1] /= hi.y - lo.y;
        if (hi.z > lo.z) o[2] /= hi.z - lo.z;
        return o[axis];
    }
};

struct Item { Box box; uint32_t value; };

struct RefNode {
    Box box;
    uint32_t child[2] = {kInvalid, kInvalid};
    std::vector<uint32_t> values;
};

struct RefBvh {
    std::vector<RefNode> nodes;
    uint32_t root = kInvalid;
};

TreeDump dump_tree(const RefBvh& b)
{
    TreeDump t;
    for (const RefNode& n : b.nodes) {
        t.boxes.insert(t.boxes.end(), {n.box.lo.x, n.box.lo.y, n.box.lo.z, n.box.hi.x, n.box.hi.y, n.box.hi.z});
        const bool leaf = n.child[0] == kInvalid && n.child[1] == kInvalid;
        t.links.insert(t.links.end(), {n.child[0], n.child[1], leaf ? (uint32_t)t.values.size() : 0u,
                                       leaf ? (uint32_t)n.values.size() : 0u});
        t.values.insert(t.values.end(), n.values.begin(), n.values.end());
    }
    return t;
}

int longest_axis(const float s[3])
{
    const float a = std::fabs(s[0]), b = std::fabs(s[1]), c = std::fabs(s[2]);
    if (a >= b && a >= c) return 0;
    if (b >= a && b >= c) return 1;
    return 2;
}

class SahBuilder {
public:
    explicit SahBuilder(RefBvh& out) : bvh_(out) {}

    void build(std::vector<Item>& items)
    {
        bvh_.root = split(items.begin(), items.end(), 32u);
    }

private:
    using It = std::vector<Item>::iterator;

    static uint32_t bucket(const Box& cb, int axis, const Item& it)
    {
        uint32_t b = (uint32_t)(12.0f * cb.offset(it.box.center(), axis));
        return b == 12 ? 11 : b;
    }

    It partition(It start, It end)
    {
        if (start == end) return end;
        Box cb;
        for (It i = start; i != end; ++i) cb.grow(i->box.center());
        float s[3];
        cb.sides(s);
        const int axis = longest_axis(s);

        uint32_t count[12] = {};
        Box bounds[12];
        for (It i = start; i < end; ++i) {
            const uint32_t b = bucket(cb, axis, *i);
            count[b]++;
            bounds[b].grow(i->box);
        }
        const float leaf_cost = (float)std::distance(start, end);
        float cost[11];
        for (uint32_t i = 0; i < 11; ++i) {
            Box b0, b1;
            uint32_t c0 = 0, c1 = 0;
            for (uint32_t j = 0; j <= i; ++j) { b0.grow(bounds[j]); c0 += count[j]; }
            for (uint32_t j = i + 1; j < 12; ++j) { b1.grow(bounds[j]); c1 += count[j]; }
            cost[i] = .125f + ((float)c0 * b0.area() + (float)c1 * b1.area()) / (leaf_cost * cb.area());
        }
        const float* m = std::min_element(&cost[0], &cost[11]);
        const uint32_t split_bucket = (uint32_t)(m - &cost[0]);
        if (leaf_cost > 2 || *m < leaf_cost)
            return std::partition(start, end, [&](const Item& it) { return bucket(cb, axis, it) <= split_bucket; });
        return end;
    }

    uint32_t split(It start, It end, uint32_t depth)
    {
        if (start == end) return kInvalid;
        RefNode n;
        for (It i = start; i != end; ++i) n.box.grow(i->box);
        const It pivot = partition(start, end);
        if (depth == 0 || pivot == end || std::distance(start, end) == 2) {
            for (It i = start; i != end; ++i) n.values.push_back(i->value);
            return push(std::move(n));
        }
        n.child[0] = split(start, pivot, depth - 1);
        n.child[1] = split(pivot, end, depth - 1);
        return push(std::move(n));
    }

    uint32_t push(RefNode&& n)
    {
        bvh_.nodes.push_back(std::move(n));
        return (uint32_t)bvh_.nodes.size() - 1;
    }

    RefBvh& bvh_;
};

// A 32-bin SAH over the instances' tight boxes for the near-first walk: every
// split is priced by area x count on both sides, leaves hold one instance
// unless all centroids coincide.  Its topology is free (the walk breaks ties by
// the reference's ranks), so it only has to prune well.
class BinnedSahBuilder {
public:
    explicit BinnedSahBuilder(RefBvh& out) : bvh_(out) {}
    void build(std::vector<Item>& items) { bvh_.root = split(items.begin(), items.end()); }

private:
    using It = std::vector<Item>::iterator;
    static constexpr int kBins = 32;

    static float centre(const Item& it, int a)
    {
        const V4 c = it.box.center();
        return a == 0 ? c.x : (a == 1 ? c.y : c.z);
    }

    uint32_t split(It start, It end)
    {
        if (start == end) return kInvalid;
        RefNode n;
        float lo[3] = {kInf, kInf, kInf}, hi[3] = {-kInf, -kInf, -kInf};
        for (It i = start; i != end; ++i) {
            n.box.grow(i->box);
            for (int a = 0; a < 3; ++a) {
                lo[a] = std::min(lo[a], centre(*i, a));
                hi[a] = std::max(hi[a], centre(*i, a));
            }
        }
        const size_t count = (size_t)std::distance(start, end);
        int best_axis = -1, best_bin = 0;
        float best_cost = kInf;
        if (count > 1) {
            for (int a = 0; a < 3; ++a) {
                const float extent = hi[a] - lo[a];
                if (!(extent > 0.0f)) continue;
                uint32_t cnt[kBins] = {};
                Box bb[kBins];
                for (It i = start; i != end; ++i) {
                    const int b = std::min(kBins - 1, (int)((float)kBins * (centre(*i, a) - lo[a]) / extent));
                    cnt[b]++;
                    bb[b].grow(i->box);
                }
                float right_area[kBins];
                uint32_t right_cnt[kBins];
                Box r;
                uint32_t rc = 0;
                for (int b = kBins - 1; b > 0; --b) {
                    r.grow(bb[b]);
                    rc += cnt[b];
                    right_area[b] = rc ? r.area() : 0.0f;
                    right_cnt[b] = rc;
                }
                Box l;
                uint32_t lc = 0;
                for (int b = 0; b < kBins - 1; ++b) {
                    l.grow(bb[b]);
                    lc += cnt[b];
                    if (lc == 0 || right_cnt[b + 1] == 0) continue;
                    const float cost = l.area() * (float)lc + right_area[b + 1] * (float)right_cnt[b + 1];
                    if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = b; }
                }
            }
        }
        It mid = end;
        if (best_axis >= 0) {
            const int a = best_axis;
            const float extent = hi[a] - lo[a];
            mid = std::partition(start, end, [&](const Item& it) {
                return std::min(kBins - 1, (int)((float)kBins * (centre(it, a) - lo[a]) / extent)) <= best_bin;
            });
        }
        if (mid == start || mid == end) {   // one instance, or all centroids in one place: a leaf
            for (It i = start; i != end; ++i) n.values.push_back(i->value);
            bvh_.nodes.push_back(std::move(n));
            return (uint32_t)bvh_.nodes.size() - 1;
        }
        n.child[0] = split(start, mid);
        n.child[1] = split(mid, end);
        bvh_.nodes.push_back(std::move(n));
        return (uint32_t)bvh_.nodes.size() - 1;
    }

    RefBvh& bvh_;
};

// Flattens a reference-topology BVH into GpuNodes; `place` appends a leaf's
// items to the item array and returns the position of the first.
template <class Place>
class Flattener {
public:
    Flattener(const RefBvh& b, std::vector<GpuNode>& nodes, Place place) : b_(b), nodes_(nodes), place_(place) {}

    uint32_t emit(uint32_t ni)
    {
        const RefNode& n = b_.nodes[ni];
        if (!n.values.empty()) {
            const uint32_t first = place_(n.values);
            return chain(first, (uint32_t)n.values.size(), n.box);
        }
        const uint32_t slot = (uint32_t)nodes_.size();
        nodes_.push_back(GpuNode{});
        uint32_t refs[2];
        const Box* boxes[2] = {nullptr, nullptr};
        for (int c = 0; c < 2; ++c) {
            if (n.child[c] == kInvalid) {
                refs[c] = PICO_REF_EMPTY;
            } else {
                refs[c] = emit(n.child[c]);
                boxes[c] = &b_.nodes[n.child[c]].box;
            }
        }
        set(slot, boxes[0], boxes[1], refs[0], refs[1]);
        return slot;
    }

private:
    uint32_t chain(uint32_t first, uint32_t count, const Box& box)
    {
        if (count <= PICO_LEAF_MAX) return pico_leaf_ref(first, count);
        const uint32_t slot = (uint32_t)nodes_.size();
        nodes_.push_back(GpuNode{});
        const uint32_t rest = chain(first + PICO_LEAF_MAX, count - PICO_LEAF_MAX, box);
        set(slot, &box, &box, pico_leaf_ref(first, PICO_LEAF_MAX), rest);
        return slot;
    }

    void set(uint32_t slot, const Box* b0, const Box* b1, uint32_t r0, uint32_t r1)
    {
        const float nan = std::numeric_limits<float>::quiet_NaN();
        GpuNode& g = nodes_[slot];
        g.c0lox = b0 ? b0->lo.x : nan; g.c0hix = b0 ? b0->hi.x : nan;
        g.c0loy = b0 ? b0->lo.y : nan; g.c0hiy = b0 ? b0->hi.y : nan;
        g.c0loz = b0 ? b0->lo.z : nan; g.c0hiz = b0 ? b0->hi.z : nan;
        g.c1lox = b1 ? b1->lo.x : nan; g.c1hix = b1 ? b1->hi.x : nan;
        g.c1loy = b1 ? b1->lo.y : nan; g.c1hiy = b1 ? b1->hi.y : nan;
        g.c1loz = b1 ? b1->lo.z : nan; g.c1hiz = b1 ? b1->hi.z : nan;
        g.ref0 = r0; g.ref1 = r1; g.pad0 = g.pad1 = 0;
    }

    const RefBvh& b_;
    std::vector<GpuNode>& nodes_;
    Place place_;
};

template <class Place>
uint32_t flatten(const RefBvh& b, std::vector<GpuNode>& nodes, Place place)
{
    if (b.root == kInvalid) return PICO_REF_EMPTY;
    Flattener<Place> f(b, nodes, place);
    return f.emit(b.root);
}

// glm mat4 * vec4: (c0*x + c1*y) + (c2*z + c3*w) per row.
V4 mul(const float* m, const V4& v)
{
    auto row = [&](int r) {
        return (m[0 * 4 + r] * v.x + m[1 * 4 + r] * v.y) + (m[2 * 4 + r] * v.z + m[3 * 4 + r] * v.w);
    };
    return {row(0), row(1), row(2), row(3)};
}

// AABB::operator*(mat4): 8 corners, divided by w, min/max from +-1e7.
Box transform_box(const Box& b, const float* m)
{
    const V4 c[8] = {b.lo,
                     {b.lo.x, b.lo.y, b.hi.z, 1.0f}, {b.hi.x, b.lo.y, b.hi.z, 1.0f}, {b.hi.x, b.lo.y, b.lo.z, 1.0f},
                     {b.lo.x, b.hi.y, b.lo.z, 1.0f}, {b.lo.x, b.hi.y, b.hi.z, 1.0f}, b.hi,
                     {b.hi.x, b.hi.y, b.lo.z, 1.0f}};
    Box r;
    r.lo = {10000000.0f, 10000000.0f, 10000000.0f, 10000000.0f};
    r.hi = {-10000000.0f, -10000000.0f, -10000000.0f, -10000000.0f};
    for (const V4& p0 : c) {
        V4 p = mul(m, p0);
        const float w = p.w;
        p = {p.x / w, p.y / w, p.z / w, p.w / w};
        r.grow(p);
    }
    return r;
}

float dot3(const float* a, const float* b) { return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2]; }
float length3(const float* a) { return std::sqrt(dot3(a, a)); }

// LowerLevelMeshBVH::generate_sampling_data's per-triangle weight
// (Core/LowerLevelMeshBVH.cpp:92-117): base * sin(acos(cos) * 180/pi) * |bc| / 2.
float triangle_weight(const float* a, const float* b, const float* c)
{
    const float ac[3] = {a[0] - c[0], a[1] - c[1], a[2] - c[2]};
    const float bc[3] = {b[0] - c[0], b[1] - c[1], b[2] - c[2]};
    const float bc_len = length3(bc);
    const float base = length3(ac);
    const float iac = 1.0f / std::sqrt(dot3(ac, ac)), ibc = 1.0f / std::sqrt(dot3(bc, bc));
    const float nac[3] = {ac[0] * iac, ac[1] * iac, ac[2] * iac};
    const float nbc[3] = {bc[0] * ibc, bc[1] * ibc, bc[2] * ibc};
    const float theta = (float)std::sin((double)std::acos(dot3(nac, nbc)) * (180.0f / 3.14159265358979323846));
    const float height = theta * bc_len;
    return (base * height) / 2.0f;
}

// Util::AliasTable::build_table (Util/AliasTable.cpp:12-87).
void alias_build(const std::vector<float>& w, std::vector<float>& bw, std::vector<uint32_t>& ba)
{
    const uint32_t n = (uint32_t)w.size();
    double acc = 0.0;
    for (float x : w) acc = acc + (double)x;
    const float total = (float)acc;
    bw.assign(n, 0.0f);
    ba.assign(n, 0u);
    for (uint32_t i = 0; i < n; ++i) bw[i] = w[i] / total;
    struct Outcome { float p; uint32_t i; };
    std::vector<Outcome> over, under;
    for (uint32_t i = 0; i < n; ++i) {
        const float p = bw[i] * (float)n;
        (p < 1.0f ? under : over).push_back({p, i});
    }
    while (!over.empty() && !under.empty()) {
        const Outcome ov = over.back(); over.pop_back();
        const Outcome un = under.back(); under.pop_back();
        bw[un.i] = un.p;
        ba[un.i] = ov.i;
        const float excess = un.p + ov.p - 1.0f;
        (excess < 1.0f ? under : over).push_back({excess, ov.i});
    }
    while (!under.empty()) { ba[under.back().i] = 0; bw[under.back().i] = 1.0f; under.pop_back(); }
    while (!over.empty()) { ba[over.back().i] = 0; bw[over.back().i] = 1.0f; over.pop_back(); }
}

}  // namespace

void mat4_inverse(const float* mf, float* out)
{
    float m[4][4];
    std::memcpy(m, mf, sizeof m);
    const float c00 = m[2][2] * m[3][3] - m[3][2] * m[2][3], c02 = m[1][2] * m[3][3] - m[3][2] * m[1][3];
    const float c03 = m[1][2] * m[2][3] - m[2][2] * m[1][3], c04 = m[2][1] * m[3][3] - m[3][1] * m[2][3];
    const float c06 = m[1][1] * m[3][3] - m[3][1] * m[1][3], c07 = m[1][1] * m[2][3] - m[2][1] * m[1][3];
    const float c08 = m[2][1] * m[3][2] - m[3][1] * m[2][2], c10 = m[1][1] * m[3][2] - m[3][1] * m[1][2];
    const float c11 = m[1][1] * m[2][2] - m[2][1] * m[1][2], c12 = m[2][0] * m[3][3] - m[3][0] * m[2][3];
    const float c14 = m[1][0] * m[3][3] - m[3][0] * m[1][3], c15 = m[1][0] * m[2][3] - m[2][0] * m[1][3];
    const float c16 = m[2][0] * m[3][2] - m[3][0] * m[2][2], c18 = m[1][0] * m[3][2] - m[3][0] * m[1][2];
    const float c19 = m[1][0] * m[2][2] - m[2][0] * m[1][2], c20 = m[2][0] * m[3][1] - m[3][0] * m[2][1];
    const float c22 = m[1][0] * m[3][1] - m[3][0] * m[1][1], c23 = m[1][0] * m[2][1] - m[2][0] * m[1][1];
    const float f[6][4] = {{c00, c00, c02, c03}, {c04, c04, c06, c07}, {c08, c08, c10, c11},
                           {c12, c12, c14, c15}, {c16, c16, c18, c19}, {c20, c20, c22, c23}};
    float vv[4][4];   // Vec0..Vec3
    for (int k = 0; k < 4; ++k) {
        vv[k][0] = m[1][k];
        vv[k][1] = vv[k][2] = vv[k][3] = m[0][k];
    }
    float inv[4][4];
    for (int i = 0; i < 4; ++i) {
        const float sa = (i % 2 == 0) ? 1.0f : -1.0f, sb = -sa;
        inv[0][i] = ((vv[1][i] * f[0][i] - vv[2][i] * f[1][i]) + vv[3][i] * f[2][i]) * sa;
        inv[1][i] = ((vv[0][i] * f[0][i] - vv[2][i] * f[3][i]) + vv[3][i] * f[4][i]) * sb;
        inv[2][i] = ((vv[0][i] * f[1][i] - vv[1][i] * f[3][i]) + vv[3][i] * f[5][i]) * sa;
        inv[3][i] = ((vv[0][i] * f[2][i] - vv[1][i] * f[4][i]) + vv[2][i] * f[5][i]) * sb;
    }
    const float d = (m[0][0] * inv[0][0] + m[0][1] * inv[1][0]) + (m[0][2] * inv[2][0] + m[0][3] * inv[3][0]);
    const float o = 1.0f / d;
    for (int c = 0; c < 4; ++c)
        for (int r = 0; r < 4; ++r) out[c * 4 + r] = inv[c][r] * o;
}

// For the physical estimator: per light triangle its world-space unit normal and
// the area density of a light sample, p(triangle) / world area, where p is the
// probability with which the alias table (sampled as AliasTable::sample,
// Util/AliasTable.cpp:89-104: a uniform bucket, then the bucket or its alias by
// a coin against the bucket's weight) returns the triangle.
static void light_triangle_geometry(const pico_mesh& m, const float* T, const std::vector<float>& bw,
                                    const std::vector<uint32_t>& ba, std::vector<float>& out)
{
    const size_t n = bw.size();
    std::vector<double> p(n, 0.0);
    for (size_t b = 0; b < n; ++b) {
        const double keep = std::min(1.0, std::max(0.0, (double)bw[b]));
        p[b] += keep / (double)n;
        if (ba[b] < n) p[ba[b]] += (1.0 - keep) / (double)n;
    }
    for (size_t t = 0; t < n; ++t) {
        double e[2][3];
        const float* a = m.positions + 3 * m.indices[3 * t];
        for (int k = 0; k < 2; ++k) {
            const float* q = m.positions + 3 * m.indices[3 * t + 1 + k];
            for (int r = 0; r < 3; ++r)
                e[k][r] = (double)T[0 * 4 + r] * ((double)q[0] - a[0]) + (double)T[1 * 4 + r] * ((double)q[1] - a[1]) +
                          (double)T[2 * 4 + r] * ((double)q[2] - a[2]);
        }
        const double c[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                             e[0][0] * e[1][1] - e[0][1] * e[1][0]};
        const double len = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        const double area = 0.5 * len;
        if (area > 0.0 && std::isfinite(area)) {
            out.insert(out.end(), {(float)(c[0] / len), (float)(c[1] / len), (float)(c[2] / len), (float)(p[t] / area)});
        } else {
            out.insert(out.end(), {0.0f, 0.0f, 1.0f, 0.0f});
        }
    }
}

// FlatScene::light_pick: cdf then pdf over the lights and, with `sun`, the sun.
static void light_pick_table(const pico_scene_desc& desc, const std::vector<GpuLight>& lights, bool sun,
                             std::vector<float>& out)
{
    const size_t n = lights.size(), slots = n + (sun ? 1 : 0);
    std::vector<double> pdf(slots, 0.0), power(n, 0.0);
    double total = 0.0;
    size_t ntri = 0;
    for (size_t k = 0; k < n; ++k) {
        if (lights[k].shape != PICO_SHAPE_TRIANGLES) continue;
        ++ntri;
        const pico_instance& in = desc.instances[lights[k].inst];
        const pico_mesh& m = desc.meshes[in.mesh];
        const float* T = in.transform;
        double area = 0.0;
        for (uint32_t t = 0; t < m.ntris; ++t) {
            double e[2][3];
            const float* a = m.positions + 3 * m.indices[3 * t];
            for (int j = 0; j < 2; ++j) {
                const float* q = m.positions + 3 * m.indices[3 * t + 1 + j];
                for (int r = 0; r < 3; ++r)
                    e[j][r] = (double)T[0 * 4 + r] * ((double)q[0] - a[0]) +
                              (double)T[1 * 4 + r] * ((double)q[1] - a[1]) +
                              (double)T[2 * 4 + r] * ((double)q[2] - a[2]);
            }
            const double c[3] = {e[0][1] * e[1][2] - e[0][2] * e[1][1], e[0][2] * e[1][0] - e[0][0] * e[1][2],
                                 e[0][0] * e[1][1] - e[0][1] * e[1][0]};
            area += 0.5 * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        }
        const float* le = desc.materials[in.material].emissive;
        const double p = ((double)le[0] + (double)le[1] + (double)le[2]) * area;
        power[k] = (std::isfinite(p) && p > 0.0) ? p : 0.0;
        total += power[k];
    }
    const double sun_share = sun ? 1.0 / (double)slots : 0.0;
    for (size_t k = 0; k < n; ++k) {
        if (lights[k].shape != PICO_SHAPE_TRIANGLES) continue;
        pdf[k] = (1.0 - sun_share) * (total > 0.0 ? power[k] / total : 1.0 / (double)ntri);
    }
    if (sun) pdf[n] = ntri ? sun_share : 1.0;
    out.assign(2 * slots, 0.0f);
    double acc = 0.0;
    for (size_t k = 0; k < slots; ++k) {
        acc += pdf[k];
        out[k] = (float)acc;
        out[slots + k] = (float)pdf[k];
    }
    // the last slot with a non-zero pdf closes the distribution at exactly 1
    for (size_t k = slots; k-- > 0;) {
        out[k] = 1.0f;
        if (pdf[k] > 0.0) break;
    }
}

std::string build_flat_scene(const pico_scene_desc& desc, FlatScene& fs)
{
    if (desc.nmeshes && !desc.meshes) return "meshes is NULL";
    if (desc.ninstances && !desc.instances) return "instances is NULL";
    if (desc.nmaterials && !desc.materials) return "materials is NULL";

    // ---- BLAS per mesh -------------------------------------------------------
    struct MeshRoot { uint32_t ref; Box box; uint32_t tri_base; };
    std::vector<MeshRoot> roots(desc.nmeshes);
    if (fs.keep_trees) fs.blas_trees.assign(desc.nmeshes, TreeDump{});
    for (uint32_t mi = 0; mi < desc.nmeshes; ++mi) {
        const pico_mesh& m = desc.meshes[mi];
        if (m.shape != PICO_SHAPE_TRIANGLES) {
            // the implicit assets have no BLAS: their bounds are [-0.5, 0.5]^3 with w = 1
            // (LowerLevelImplicitShapesBVH.cpp:54-57, 66-68)
            if (m.shape != PICO_SHAPE_SPHERE && m.shape != PICO_SHAPE_CUBE)
                return "mesh " + std::to_string(mi) + ": unknown shape";
            roots[mi].ref = m.shape == PICO_SHAPE_SPHERE ? PICO_REF_SPHERE : PICO_REF_CUBE;
            roots[mi].box.lo = {-0.5f, -0.5f, -0.5f, 1.0f};
            roots[mi].box.hi = {0.5f, 0.5f, 0.5f, 1.0f};
            roots[mi].tri_base = 0;
            continue;
        }
        if (m.ntris && (!m.positions || !m.normals || !m.indices)) return "mesh " + std::to_string(mi) + " lacks arrays";
        for (uint64_t k = 0; k < 3ull * m.ntris; ++k)
            if (m.indices[k] >= m.nverts) return "mesh " + std::to_string(mi) + " index out of range";
        std::vector<Item> items(m.ntris);
        for (uint32_t t = 0; t < m.ntris; ++t) {
            float lo[3] = {kInf, kInf, kInf}, hi[3] = {-kInf, -kInf, -kInf};
            for (int k = 0; k < 3; ++k) {
                const float* p = m.positions + 3 * m.indices[3 * t + k];
                for (int a = 0; a < 3; ++a) lo[a] = sel_min(lo[a], p[a]);
            }
            for (int k = 0; k < 3; ++k) {
                const float* p = m.positions + 3 * m.indices[3 * t + k];
                for (int a = 0; a < 3; ++a) hi[a] = sel_max(hi[a], p[a]);
            }
            items[t].box.lo = {lo[0], lo[1], lo[2], 1.0f};
            items[t].box.hi = {hi[0], hi[1], hi[2], 1.0f};
            items[t].value = t;
        }
        RefBvh bvh;
        SahBuilder(bvh).build(items);
        if (fs.keep_trees) fs.blas_trees[mi] = dump_tree(bvh);
        const uint32_t tri_base = (uint32_t)fs.tris.size();
        const size_t before = fs.nodes.size();
        auto place = [&](const std::vector<uint32_t>& values) -> uint32_t {
            const uint32_t first = (uint32_t)fs.tris.size();
            for (uint32_t prim : values) {
                const float* a = m.positions + 3 * m.indices[3 * prim];
                const float* b = m.positions + 3 * m.indices[3 * prim + 1];
                const float* c = m.positions + 3 * m.indices[3 * prim + 2];
                fs.tris.push_back(GpuTri{a[0], a[1], a[2], prim, b[0], b[1], b[2], tri_base, c[0], c[1], c[2], mi});
                const float* na = m.normals + 3 * m.indices[3 * prim];
                const float* nb = m.normals + 3 * m.indices[3 * prim + 1];
                const float* nc = m.normals + 3 * m.indices[3 * prim + 2];
                fs.tri_shade.push_back(GpuTriShade{na[0], na[1], na[2], 0, nb[0], nb[1], nb[2], 0, nc[0], nc[1], nc[2], 0});
            }
            return first;
        };
        roots[mi].ref = flatten(bvh, fs.nodes, place);
        roots[mi].box = bvh.root == kInvalid ? Box{} : bvh.nodes[bvh.root].box;
        roots[mi].tri_base = tri_base;
        fs.blas_nodes += (uint32_t)(fs.nodes.size() - before);
        if (fs.tris.size() > PICO_FIRST_MAX) return "too many triangles";
    }

    // ---- TLAS over instances --------------------------------------------------
    fs.inst_rank.assign(desc.ninstances, 0u);
    fs.inst_shade.resize(desc.ninstances);
    std::vector<Item> items(desc.ninstances);
    std::vector<std::array<float, 16>> inverses(desc.ninstances);
    for (uint32_t i = 0; i < desc.ninstances; ++i) {
        const pico_instance& in = desc.instances[i];
        if (in.mesh >= desc.nmeshes) return "instance " + std::to_string(i) + " names a missing mesh";
        if (in.material >= desc.nmaterials) return "instance " + std::to_string(i) + " names a missing material";
        if (in.bsdf > PICO_BSDF_DELTA) return "instance " + std::to_string(i) + ": BSRDF kind not supported";
        mat4_inverse(in.transform, inverses[i].data());
        const pico_mesh& m = desc.meshes[in.mesh];
        Box mb;   // LowerLevelBVH::get_bounds: the mesh AABB, or the implicit shape's box
        if (m.shape != PICO_SHAPE_TRIANGLES) {
            mb = roots[in.mesh].box;
        } else {
            mb.lo = {m.aabb_min[0], m.aabb_min[1], m.aabb_min[2], 1.0f};
            mb.hi = {m.aabb_max[0], m.aabb_max[1], m.aabb_max[2], 1.0f};
        }
        items[i].box = transform_box(mb, in.transform);
        items[i].value = i;
        fs.inst_shade[i] = GpuInstanceShade{in.bsdf, in.material, in.mesh, 0};
    }
    RefBvh tlas;
    SahBuilder(tlas).build(items);
    if (fs.keep_trees) fs.tlas_tree = dump_tree(tlas);
    const size_t before = fs.nodes.size();
    auto place = [&](const std::vector<uint32_t>& values) -> uint32_t {
        const uint32_t first = (uint32_t)fs.insts.size();
        for (uint32_t i : values) {
            const pico_instance& in = desc.instances[i];
            GpuInstance g{};
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 4; ++c) g.inv[r][c] = inverses[i][c * 4 + r];
            for (int r = 0; r < 4; ++r)
                for (int c = 0; c < 4; ++c) g.fwd[r][c] = in.transform[c * 4 + r];
            const MeshRoot& mr = roots[in.mesh];
            const bool empty = mr.ref == PICO_REF_EMPTY;
            const float nan = std::numeric_limits<float>::quiet_NaN();
            g.root_lo[0] = empty ? nan : mr.box.lo.x; g.root_lo[1] = empty ? nan : mr.box.lo.y;
            g.root_lo[2] = empty ? nan : mr.box.lo.z;
            g.root_hi[0] = empty ? nan : mr.box.hi.x; g.root_hi[1] = empty ? nan : mr.box.hi.y;
            g.root_hi[2] = empty ? nan : mr.box.hi.z;
            g.root_ref = mr.ref;
            g.inst_id = i;
            fs.inst_rank[i] = (uint32_t)fs.insts.size();
            fs.tlas_items.push_back((uint32_t)fs.insts.size());   // the reference tree's items are its ranks
            fs.insts.push_back(g);
        }
        return first;
    };
    fs.tlas_root_ref = flatten(tlas, fs.nodes, place);
    fs.tlas_nodes = (uint32_t)(fs.nodes.size() - before);

    // The same TLAS topology with boxes refitted to each instance's transformed
    // vertices (for the near-first walk).  Computed in double and widened by
    // 1e-5 of the scene's largest coordinate magnitude, far above the float error
    // of a hit point seen from anywhere in the scene.  Falls back to the
    // reference's box when transforming every vertex would be costly.
    uint64_t work = 0;
    for (uint32_t i = 0; i < desc.ninstances; ++i) work += desc.meshes[desc.instances[i].mesh].nverts;
    std::vector<std::array<double, 6>> extent(desc.ninstances);
    double mag = 1.0;
    for (uint32_t i = 0; i < desc.ninstances; ++i) {
        const pico_instance& in = desc.instances[i];
        const pico_mesh& m = desc.meshes[in.mesh];
        std::array<double, 6>& e = extent[i];
        e = {1e300, 1e300, 1e300, -1e300, -1e300, -1e300};
        const bool implicit = m.shape != PICO_SHAPE_TRIANGLES;   // bounded by its box's 8 corners
        if (!implicit && (work > 400000000ull || m.nverts == 0)) continue;
        static const float kCorners[8][3] = {{-0.5f, -0.5f, -0.5f}, {0.5f, -0.5f, -0.5f}, {-0.5f, 0.5f, -0.5f},
                                             {0.5f, 0.5f, -0.5f},   {-0.5f, -0.5f, 0.5f}, {0.5f, -0.5f, 0.5f},
                                             {-0.5f, 0.5f, 0.5f},   {0.5f, 0.5f, 0.5f}};
        const float* T = in.transform;
        const uint32_t nv = implicit ? 8u : m.nverts;
        for (uint32_t v = 0; v < nv; ++v) {
            const float* pv = implicit ? kCorners[v] : m.positions + 3 * v;
            const double x = pv[0], y = pv[1], z = pv[2];
            for (int r = 0; r < 3; ++r) {
                const double w = (double)T[0 * 4 + r] * x + (double)T[1 * 4 + r] * y + (double)T[2 * 4 + r] * z +
                                 (double)T[3 * 4 + r];
                e[r] = std::min(e[r], w);
                e[3 + r] = std::max(e[3 + r], w);
            }
        }
        for (int r = 0; r < 3; ++r) mag = std::max(mag, std::max(std::fabs(e[r]), std::fabs(e[3 + r])));
    }
    const double pad = 1e-5 * mag;
    std::vector<Box> tight(desc.ninstances);
    for (uint32_t i = 0; i < desc.ninstances; ++i) {
        const std::array<double, 6>& e = extent[i];
        if (!(e[0] <= e[3])) {
            tight[i] = items[i].box;
            continue;
        }
        tight[i].lo = {(float)(e[0] - pad), (float)(e[1] - pad), (float)(e[2] - pad), 1.0f};
        tight[i].hi = {(float)(e[3] + pad), (float)(e[4] + pad), (float)(e[5] + pad), 1.0f};
    }
    // the near-first TLAS: a fresh SAH over the tight boxes, leaves listing ranks
    RefBvh refit;
    {
        std::vector<Item> titems(desc.ninstances);
        for (uint32_t i = 0; i < desc.ninstances; ++i) titems[i] = Item{tight[i], fs.inst_rank[i]};
        BinnedSahBuilder(refit).build(titems);
    }
    auto list_ranks = [&](const std::vector<uint32_t>& ranks) -> uint32_t {
        const uint32_t first = (uint32_t)fs.tlas_items.size();
        fs.tlas_items.insert(fs.tlas_items.end(), ranks.begin(), ranks.end());
        return first;
    };
    fs.tlas_fast_root_ref = flatten(refit, fs.nodes, list_ranks);
    if (fs.tlas_items.size() > PICO_FIRST_MAX) return "too many instances";
    if (refit.root != kInvalid) {
        const Box& b = refit.nodes[refit.root].box;
        fs.tlas_fast_lo[0] = b.lo.x; fs.tlas_fast_lo[1] = b.lo.y; fs.tlas_fast_lo[2] = b.lo.z;
        fs.tlas_fast_hi[0] = b.hi.x; fs.tlas_fast_hi[1] = b.hi.y; fs.tlas_fast_hi[2] = b.hi.z;
    } else {
        const float nan = std::numeric_limits<float>::quiet_NaN();
        for (int a = 0; a < 3; ++a) fs.tlas_fast_lo[a] = fs.tlas_fast_hi[a] = nan;
    }
    if (tlas.root != kInvalid) {
        const Box& b = tlas.nodes[tlas.root].box;
        fs.tlas_lo[0] = b.lo.x; fs.tlas_lo[1] = b.lo.y; fs.tlas_lo[2] = b.lo.z;
        fs.tlas_hi[0] = b.hi.x; fs.tlas_hi[1] = b.hi.y; fs.tlas_hi[2] = b.hi.z;
    } else {
        const float nan = std::numeric_limits<float>::quiet_NaN();
        for (int a = 0; a < 3; ++a) fs.tlas_lo[a] = fs.tlas_hi[a] = nan;
    }

    // ---- materials ------------------------------------------------------------
    fs.materials.resize(desc.nmaterials);
    for (uint32_t i = 0; i < desc.nmaterials; ++i) {
        const pico_material& m = desc.materials[i];
        GpuMaterial g{};
        for (int a = 0; a < 3; ++a) {
            g.diffuse[a] = m.diffuse[a]; g.specular[a] = m.specular[a]; g.emissive[a] = m.emissive[a];
        }
        g.roughness = m.roughness;
        g.ior = m.index_of_refraction;
        const float s = length3(m.specular), d = length3(m.diffuse);
        g.reflectance = s / (s + d);
        fs.materials[i] = g;
    }

    // ---- NEE lights (Scene.cpp:406-412: every "Light" instance, in order) -----
    fs.light_of_inst.assign(desc.ninstances, ~0u);
    for (uint32_t i = 0; i < desc.ninstances; ++i) {
        const pico_instance& in = desc.instances[i];
        if (in.bsdf != PICO_BSDF_LIGHT) continue;
        const pico_mesh& m = desc.meshes[in.mesh];
        fs.light_of_inst[i] = (uint32_t)fs.lights.size();
        if (m.shape != PICO_SHAPE_TRIANGLES) {   // sampled by the shape itself (sample_geometry)
            fs.lights.push_back(GpuLight{i, 0, 0, m.shape});
            continue;
        }
        if (m.ntris == 0) return "light instance " + std::to_string(i) + " has an empty mesh";
        GpuLight l{i, (uint32_t)fs.light_alias_weight.size(), m.ntris, PICO_SHAPE_TRIANGLES};
        std::vector<float> w(m.ntris);
        for (uint32_t t = 0; t < m.ntris; ++t) {
            const float* a = m.positions + 3 * m.indices[3 * t];
            const float* b = m.positions + 3 * m.indices[3 * t + 1];
            const float* c = m.positions + 3 * m.indices[3 * t + 2];
            w[t] = triangle_weight(a, b, c);
            for (const float* p : {a, b, c}) fs.light_positions.insert(fs.light_positions.end(), p, p + 3);
        }
        std::vector<float> bw;
        std::vector<uint32_t> ba;
        alias_build(w, bw, ba);
        light_triangle_geometry(m, in.transform, bw, ba, fs.light_tri_geo);
        fs.light_alias_weight.insert(fs.light_alias_weight.end(), bw.begin(), bw.end());
        fs.light_alias_index.insert(fs.light_alias_index.end(), ba.begin(), ba.end());
        fs.lights.push_back(l);
    }
    // World boxes of the NEE lights, for the early exit of the closest-hit shadow
    // rays: every point a hit on a light reports (T times an object-space point of
    // its triangles, or of its implicit shape's unit box) lies in its light's box up
    // to float error, so no hit on a light lies nearer than the nearest box.  The
    // boxes are widened by 1e-4 of the scene's largest coordinate magnitude, ten
    // times the near-first TLAS's widening.  None when a light's vertices were not
    // transformed, a box is not finite, or there are too many lights to scan per ray.
    fs.light_boxes.clear();
    fs.light_bounds = fs.lights.size() <= kMaxBoundedLights;
    const double lpad = 1e-4 * mag;
    for (size_t l = 0; fs.light_bounds && l < fs.lights.size(); ++l) {
        const std::array<double, 6>& e = extent[fs.lights[l].inst];
        bool ok = e[0] <= e[3] && e[1] <= e[4] && e[2] <= e[5];
        for (int a = 0; a < 6; ++a) ok = ok && std::isfinite(e[a]);
        if (!ok) {
            fs.light_bounds = false;
            break;
        }
        for (int a = 0; a < 3; ++a) fs.light_boxes.push_back((float)(e[a] - lpad));
        fs.light_boxes.push_back(0.0f);
        for (int a = 0; a < 3; ++a) fs.light_boxes.push_back((float)(e[3 + a] + lpad));
        fs.light_boxes.push_back(0.0f);
    }
    if (!fs.light_bounds) fs.light_boxes.clear();

    for (int a = 0; a < 3; ++a) fs.sky[a] = desc.sky_rgb[a];
    const bool sun = desc.sky && desc.sky->use_sun;
    light_pick_table(desc, fs.lights, sun, fs.light_pick);

    // ---- sky image and sun (Scene::process_globals, Core/Scene.cpp:639-700) -----
    if (const pico_sky* k = desc.sky) {
        fs.sky_kind = k->kind;
        if (k->kind == PICO_SKY_CUBE_RGBA8 || k->kind == PICO_SKY_EQUIRECT_RGBAF) {
            if (!k->pixels || k->width == 0 || k->height == 0) return "sky image without pixels";
            const size_t texels = (size_t)k->width * k->height * (k->kind == PICO_SKY_CUBE_RGBA8 ? 6 : 1);
            const size_t bytes = texels * (k->kind == PICO_SKY_CUBE_RGBA8 ? 4 : 16);
            const unsigned char* p = static_cast<const unsigned char*>(k->pixels);
            fs.sky_pixels.assign(p, p + bytes);
            fs.sky_w = k->width;
            fs.sky_h = k->height;
        } else if (k->kind != PICO_SKY_CONSTANT) {
            return "unknown sky kind " + std::to_string(k->kind);
        }
        fs.use_sun = k->use_sun ? 1u : 0u;
        for (int a = 0; a < 3; ++a) {
            fs.sun_dir[a] = k->sun_direction[a];
            fs.sun_col[a] = k->sun_colour[a];
        }
    }
    return std::string();
}

}  // namespace pico
