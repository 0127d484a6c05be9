// Reference harness (test infrastructure only).
//
// Links the Pico reference's own sources (compiled unmodified from the Pico
// tree by oracle/Makefile) and exposes their hot-path routines through a C
// interface, so that golden vectors can be generated from the reference itself
// and the reference CPU tracer can be timed.  Scenes are assembled in memory in
// a fixed order, as Scene::add_mesh_instance does (Core/Scene.cpp:321-422),
// without the JSON/assimp file loaders.
//
// Closest-hit IDs are recovered through the reference's public API only: each
// mesh is handed to LowerLevelMeshBVH un-indexed, with every triangle's three
// vertices coloured (prim, 0, 0, 1) and given the UVs (0,0), (1,0), (0,1), so
// the interpolated fragment carries the primitive index in its colour and the
// barycentrics (u, v) in its UV.  Positions are unchanged, so the BVH and the
// ray/triangle arithmetic are exactly those of the indexed mesh.  The instance
// index comes from the BSRDF pointer, which is unique per TLAS entry.
//
// Private members (BVH node arrays, alias buckets) are read for introspection
// with the explicit-instantiation access idiom; no reference code is changed.

#include "Core/Camera.hpp"
#include "Core/Image.hpp"
#include "Core/LowerLevelImplicitShapesBVH.hpp"
#include "Core/LowerLevelMeshBVH.hpp"
#include "Core/MaterialManager.hpp"
#include "Core/RandUtils.hpp"
#include "Core/Scene.hpp"
#include "Core/ThreadPool.hpp"
#include "Core/UpperLevelBVH.hpp"
#include "Core/vectorUtils.hpp"
#include "Render/BasicMaterials.hpp"
#include "Render/BSRDF.hpp"
#include "Render/Distributions.hpp"
#include "Render/Integrators.hpp"
#include "Util/AliasTable.hpp"
#include "Util/Denoisers.hpp"
#include "Util/Tiler.hpp"
#include "Util/ToneMappers.hpp"

#include "assimp/mesh.h"
#include "stbi_image_write.h"
#include "glm/ext.hpp"   // as Core/Scene.cpp:24 (brings gtx/scalar_multiplication)

#include "../pico_oracle.h"

#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <random>
#include <vector>

using namespace Core::Acceleration_Structures;

namespace {

// ---- explicit-instantiation access idiom ------------------------------------
template <class Tag, auto M> struct Robber { friend auto robbed(Tag) { return M; } };

struct TlasTag { friend auto robbed(TlasTag); };
template struct Robber<TlasTag, &UpperLevelBVH::m_acceleration_structure>;
struct EntriesTag { friend auto robbed(EntriesTag); };
template struct Robber<EntriesTag, &UpperLevelBVH::mLowerLevelBVHs>;
struct BlasTag { friend auto robbed(BlasTag); };
template struct Robber<BlasTag, &LowerLevelMeshBVH::m_acceleration_structure>;
struct AreaTag { friend auto robbed(AreaTag); };
template struct Robber<AreaTag, &LowerLevelMeshBVH::m_triangle_area>;
struct AliasTag { friend auto robbed(AliasTag); };
template struct Robber<AliasTag, &LowerLevelMeshBVH::m_aliasTable>;
struct BucketsTag { friend auto robbed(BucketsTag); };
template struct Robber<BucketsTag, &Util::AliasTable::m_buckets>;
struct TNodesTag { friend auto robbed(TNodesTag); };
template struct Robber<TNodesTag, &BVH<const UpperLevelBVH::Entry*, 2>::m_nodes>;
struct TRootTag { friend auto robbed(TRootTag); };
template struct Robber<TRootTag, &BVH<const UpperLevelBVH::Entry*, 2>::m_root>;
struct BNodesTag { friend auto robbed(BNodesTag); };
template struct Robber<BNodesTag, &BVH<uint32_t, 2>::m_nodes>;
struct BRootTag { friend auto robbed(BRootTag); };
template struct Robber<BRootTag, &BVH<uint32_t, 2>::m_root>;

// A constant material returning a fixed EvaluatedMaterial.
class FixedMaterial : public Core::Material {
public:
    explicit FixedMaterial(const po_material& m)
    {
        e.diffuse = glm::vec3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
        e.specular = glm::vec3(m.specular[0], m.specular[1], m.specular[2]);
        e.roughness = m.roughness;
        e.normal = glm::vec3(0.0f, 1.0f, 0.0f);
        e.emissive = glm::vec3(m.emissive[0], m.emissive[1], m.emissive[2]);
    }
    Core::EvaluatedMaterial evaluate_material(const glm::vec2&) const override { return e; }
    bool is_light() const override { return e.emits_light(); }
    size_t get_residence_size() const override { return 0; }
    bool is_resident() const override { return true; }
    void make_resident(void*) override {}
    void make_nonresident() override {}
private:
    Core::EvaluatedMaterial e;
};

// A constant transparent material (what Scene::add_material makes for an
// "IndexOfRefraction" entry, Core/Scene.cpp:526-530), fixed EvaluatedMaterial.
class FixedTransparentMaterial : public Render::ConstantTransparentMaterial {
public:
    explicit FixedTransparentMaterial(const po_material& m) : Render::ConstantTransparentMaterial(1.0f, m.index_of_refraction)
    {
        e.diffuse = glm::vec3(m.diffuse[0], m.diffuse[1], m.diffuse[2]);
        e.specular = glm::vec3(m.specular[0], m.specular[1], m.specular[2]);
        e.roughness = m.roughness;
        e.normal = glm::vec3(0.0f, 1.0f, 0.0f);
        e.emissive = glm::vec3(m.emissive[0], m.emissive[1], m.emissive[2]);
    }
    Core::EvaluatedMaterial evaluate_material(const glm::vec2&) const override { return e; }
    bool is_light() const override { return e.emits_light(); }
private:
    Core::EvaluatedMaterial e;
};

struct RefScene {
    std::vector<std::unique_ptr<LowerLevelBVH>> blas;
    std::vector<uint32_t> shape;
    UpperLevelBVH tlas;
    Core::MaterialManager materials;
    std::vector<Scene::Light> lights;
    std::unique_ptr<Core::ImageCube> sky;
    Scene::Sun sun{};
    std::map<const Render::BSRDF*, uint32_t> instance_of;
    std::vector<uint32_t> ntris;
};

glm::mat4 to_mat4(const float* m)
{
    glm::mat4 r;
    std::memcpy(&r[0][0], m, sizeof(float) * 16);
    return r;
}

Scene::Camera to_camera(const po_camera* c)
{
    Scene::Camera cam(glm::vec3(c->position[0], c->position[1], c->position[2]),
                      glm::vec3(c->direction[0], c->direction[1], c->direction[2]), c->aspect,
                      c->near_plane, c->far_plane, c->fov);
    cam.setUp(glm::vec3(c->up[0], c->up[1], c->up[2]));
    cam.set_resolution(glm::uvec2(c->resolution[0], c->resolution[1]));
    return cam;
}

std::unique_ptr<Render::BSRDF> make_bsrdf(RefScene& s, uint32_t kind, uint32_t material)
{
    std::unique_ptr<Render::BSRDF> b;
    if (kind == PO_DIFFUSE) {
        std::unique_ptr<Render::Distribution> d = std::make_unique<Render::Cos_Weighted_Hemisphere_Distribution>();
        b = std::make_unique<Render::Diffuse_BRDF>(d, s.materials, material);
    } else if (kind == PO_SPECULAR) {
        std::unique_ptr<Render::Distribution> d = std::make_unique<Render::Beckmann_All_Microfacet_Distribution>();
        b = std::make_unique<Render::Specular_BRDF>(d, s.materials, material);
    } else if (kind == PO_DIELECTRIC) {
        std::unique_ptr<Render::Distribution> d0 = std::make_unique<Render::Cos_Weighted_Hemisphere_Distribution>();
        std::unique_ptr<Render::Distribution> d1 = std::make_unique<Render::Beckmann_All_Microfacet_Distribution>();
        b = std::make_unique<Render::Dielectric_BRDF>(d0, d1, s.materials, material);
    } else if (kind == PO_LIGHT) {
        b = std::make_unique<Render::Light_BRDF>(s.materials, material);
    } else if (kind == PO_BTDF) {                                 // "Transparent", Scene.cpp:392-398
        std::unique_ptr<Render::Distribution> d = std::make_unique<Render::Beckmann_All_Microfacet_Distribution>();
        b = std::make_unique<Render::Transparent_BTDF>(d, s.materials, material);
    } else if (kind == PO_FRESNEL) {                              // "Fresnel", Scene.cpp:399-405
        std::unique_ptr<Render::Distribution> d0 = std::make_unique<Render::Beckmann_All_Microfacet_Distribution>();
        std::unique_ptr<Render::Distribution> d1 = std::make_unique<Render::Beckmann_All_Microfacet_Distribution>();
        b = std::make_unique<Render::Fresnel_BTDF>(d0, d1, s.materials, material);
    } else if (kind == PO_DELTA) {                                // "Delta", Scene.cpp:413-416
        b = std::make_unique<Render::Specular_Delta_BRDF>(s.materials, material);
    }
    return b;
}

// The triangle index carried in the vertex colour; implicit shapes have none.
uint32_t prim_of(const RefScene& s, uint32_t inst, const InterpolatedVertex& v)
{
    return s.shape[inst] != PO_SHAPE_TRIANGLES ? PO_IMPLICIT_PRIM : (uint32_t)std::lround(v.mVertexColour.x);
}

void fill_fragment(const RefScene& s, const InterpolatedVertex& v, float t_world, po_fragment* f)
{
    f->inst = s.instance_of.at(v.m_bsrdf);
    f->prim = prim_of(s, f->inst, v);
    f->t = t_world;
    f->u = v.mUV.x;
    f->v = v.mUV.y;
    f->position[0] = v.mPosition.x; f->position[1] = v.mPosition.y;
    f->position[2] = v.mPosition.z; f->position[3] = v.mPosition.w;
    f->normal[0] = v.mNormal.x; f->normal[1] = v.mNormal.y; f->normal[2] = v.mNormal.z;
    f->uv[0] = v.mUV.x; f->uv[1] = v.mUV.y;
}

Core::Ray to_ray(const po_ray& r)
{
    Core::Ray ray{};
    ray.mOrigin = glm::vec4(r.org[0], r.org[1], r.org[2], r.org[3]);
    ray.mDirection = glm::vec3(r.dir[0], r.dir[1], r.dir[2]);
    ray.mLenght = r.dir[3];
    return ray;
}

void trace_one(const RefScene& s, const po_ray& r, po_fragment* f)
{
    Core::Ray ray = to_ray(r);
    InterpolatedVertex v{};
    std::memset(f, 0, sizeof(*f));
    if (s.tlas.get_closest_intersection(ray, &v)) {
        // the same world distance lower_level_intersector::intersects returns
        const float t = glm::length(v.mPosition - ray.mOrigin);
        fill_fragment(s, v, t, f);
    } else {
        f->inst = f->prim = 0xffffffffu;
        f->t = INFINITY;
    }
}

template <class B> void dump_nodes(const B* bvh, uint32_t root, float* boxes, uint32_t* links,
                                   uint32_t* values, const std::vector<UpperLevelBVH::Entry>* entries)
{
    (void)root;
    uint32_t nv = 0;
    const auto& nodes = bvh->*robbed(std::conditional_t<std::is_same_v<B, BVH<uint32_t, 2>>, BNodesTag, TNodesTag>{});
    for (size_t i = 0; i < nodes.size(); ++i) {
        const auto& n = nodes[i];
        if (boxes) {
            float* o = boxes + 6 * i;
            o[0] = n.m_bounding_box.get_min().x; o[1] = n.m_bounding_box.get_min().y;
            o[2] = n.m_bounding_box.get_min().z; o[3] = n.m_bounding_box.get_max().x;
            o[4] = n.m_bounding_box.get_max().y; o[5] = n.m_bounding_box.get_max().z;
        }
        if (links) {
            uint32_t* l = links + 4 * i;
            l[0] = n.m_children[0]; l[1] = n.m_children[1];
            l[2] = n.m_values.empty() ? 0u : nv; l[3] = (uint32_t)n.m_values.size();
        }
        for (const auto& val : n.m_values) {
            if (values) {
                if constexpr (std::is_same_v<B, BVH<uint32_t, 2>>)
                    values[nv] = val.m_value;
                else
                    values[nv] = (uint32_t)(val.m_value - entries->data());
            }
            ++nv;
        }
    }
}

} // namespace

extern "C" {

void* ref_scene_create(const po_mesh_desc* meshes, uint32_t nmeshes, const po_instance_desc* inst,
                       uint32_t ninst, const po_material* mats, uint32_t nmats)
{
    auto* s = new RefScene();
    for (uint32_t m = 0; m < nmeshes; ++m) {
        const po_mesh_desc& d = meshes[m];
        if (d.shape == PO_SHAPE_SPHERE || d.shape == PO_SHAPE_CUBE) {   // Scene.cpp:49-57
            if (d.shape == PO_SHAPE_SPHERE) s->blas.push_back(std::make_unique<LowerLevelSphereBVH>(0.5f));
            else s->blas.push_back(std::make_unique<LowerLevelCube>());
            s->ntris.push_back(0);
            continue;
        }
        aiMesh mesh;
        mesh.mName = aiString("mesh");
        mesh.mNumVertices = 3 * d.ntris;
        mesh.mNumFaces = d.ntris;
        mesh.mVertices = new aiVector3D[3 * d.ntris];
        mesh.mNormals = new aiVector3D[3 * d.ntris];
        mesh.mTextureCoords[0] = new aiVector3D[3 * d.ntris];
        mesh.mNumUVComponents[0] = 2;
        mesh.mColors[0] = new aiColor4D[3 * d.ntris];
        mesh.mFaces = new aiFace[d.ntris];
        static const float kUV[3][2] = {{0, 0}, {1, 0}, {0, 1}};
        for (uint32_t t = 0; t < d.ntris; ++t) {
            mesh.mFaces[t].mNumIndices = 3;
            mesh.mFaces[t].mIndices = new unsigned int[3];
            for (int k = 0; k < 3; ++k) {
                const uint32_t src = d.indices[3 * t + k], dst = 3 * t + k;
                mesh.mFaces[t].mIndices[k] = dst;
                mesh.mVertices[dst] = aiVector3D(d.positions[3 * src], d.positions[3 * src + 1], d.positions[3 * src + 2]);
                mesh.mNormals[dst] = aiVector3D(d.normals[3 * src], d.normals[3 * src + 1], d.normals[3 * src + 2]);
                mesh.mTextureCoords[0][dst] = aiVector3D(kUV[k][0], kUV[k][1], 0.0f);
                mesh.mColors[0][dst] = aiColor4D((float)t, 0.0f, 0.0f, 1.0f);
            }
        }
        mesh.mAABB.mMin = aiVector3D(d.aabb_min[0], d.aabb_min[1], d.aabb_min[2]);
        mesh.mAABB.mMax = aiVector3D(d.aabb_max[0], d.aabb_max[1], d.aabb_max[2]);
        s->blas.push_back(std::make_unique<LowerLevelMeshBVH>(&mesh));
        s->ntris.push_back(d.ntris);
    }
    for (uint32_t i = 0; i < nmats; ++i) {
        std::unique_ptr<Core::Material> m;
        if (mats[i].index_of_refraction > 0.0f) m = std::make_unique<FixedTransparentMaterial>(mats[i]);
        else m = std::make_unique<FixedMaterial>(mats[i]);
        s->materials.add_material(m);
    }
    std::vector<bool> sampled(nmeshes, false);
    for (uint32_t i = 0; i < ninst; ++i) {
        const glm::mat4 T = to_mat4(inst[i].transform);
        std::unique_ptr<Render::BSRDF> b = make_bsrdf(*s, inst[i].bsdf, inst[i].material);
        if (inst[i].bsdf == PO_LIGHT) {                      // Scene.cpp:406-412
            if (!sampled[inst[i].mesh]) s->blas[inst[i].mesh]->generate_sampling_data();
            sampled[inst[i].mesh] = true;
            s->lights.push_back({T, glm::inverse(T), s->blas[inst[i].mesh].get()});
        }
        s->instance_of[b.get()] = i;
        s->shape.push_back(meshes[inst[i].mesh].shape);
        s->tlas.add_lower_level_bvh(s->blas[inst[i].mesh].get(), T, b);
    }
    s->tlas.build();
    unsigned char* black = static_cast<unsigned char*>(malloc(24));   // Scene.cpp:683-690
    std::memset(black, 0, 24);
    s->sky = std::make_unique<Core::ImageCube>(black, Core::ImageExtent{1, 1, 1}, Core::Format::kRBGA_8UNorm);
    s->sun.m_sky_box = s->sky.get();
    s->sun.m_use_sun = false;
    s->sun.m_sun_direction = glm::vec3(0.0f, -1.0f, 0.0f);
    s->sun.m_sun_colour = glm::vec3(1.0f);
    return s;
}

void ref_scene_destroy(void* p) { delete static_cast<RefScene*>(p); }

}  // extern "C"

// The ImageCube Scene::process_globals builds for a sky (Scene.cpp:639-690): six
// RGBA8 faces, one RGBA float HDRI, or a 1x1 RGBA float image of a constant colour.
static std::unique_ptr<Core::ImageCube> make_sky(const po_sky* sky, const float* rgb)
{
    if (sky && sky->kind == PO_SKY_CUBE_RGBA8) {
        const size_t n = (size_t)6 * sky->width * sky->height * 4;
        unsigned char* data = static_cast<unsigned char*>(malloc(n));
        std::memcpy(data, sky->pixels, n);
        return std::make_unique<Core::ImageCube>(data, Core::ImageExtent{sky->width, sky->height, 6},
                                                 Core::Format::kRBGA_8UNorm);
    }
    if (sky && sky->kind == PO_SKY_EQUIRECT_RGBAF) {
        const size_t n = (size_t)sky->width * sky->height * 4 * sizeof(float);
        unsigned char* data = static_cast<unsigned char*>(malloc(n));
        std::memcpy(data, sky->pixels, n);
        return std::make_unique<Core::ImageCube>(data, Core::ImageExtent{sky->width, sky->height, 1},
                                                 Core::Format::kRGBA_F);
    }
    float* data = static_cast<float*>(malloc(4 * sizeof(float)));
    for (int c = 0; c < 3; ++c) data[c] = rgb ? rgb[c] : 0.0f;
    data[3] = 0.0f;
    return std::make_unique<Core::ImageCube>(reinterpret_cast<unsigned char*>(data), Core::ImageExtent{1, 1, 1},
                                             Core::Format::kRGBA_F);
}

extern "C" {

void ref_scene_set_sky(void* p, const po_sky* sky, const float* rgb)
{
    auto* s = static_cast<RefScene*>(p);
    s->sky = make_sky(sky, rgb);
    s->sun.m_sky_box = s->sky.get();
    s->sun.m_use_sun = sky && sky->use_sun;
    if (sky) {
        s->sun.m_sun_direction = glm::vec3(sky->sun_direction[0], sky->sun_direction[1], sky->sun_direction[2]);
        s->sun.m_sun_colour = glm::vec3(sky->sun_colour[0], sky->sun_colour[1], sky->sun_colour[2]);
    }
}

void ref_sky_sample(const po_sky* sky, const float* dirs, uint32_t n, float* rgba)
{
    const std::unique_ptr<Core::ImageCube> cube = make_sky(sky, nullptr);
    for (uint32_t i = 0; i < n; ++i) {
        const glm::vec4 c = cube->sample4(glm::vec3(dirs[3 * i], dirs[3 * i + 1], dirs[3 * i + 2]));
        rgba[4 * i] = c.x; rgba[4 * i + 1] = c.y; rgba[4 * i + 2] = c.z; rgba[4 * i + 3] = c.w;
    }
}

void ref_trace(const void* p, const po_ray* rays, uint32_t n, po_fragment* out)
{
    const auto* s = static_cast<const RefScene*>(p);
    for (uint32_t i = 0; i < n; ++i) trace_one(*s, rays[i], &out[i]);
}

// UpperLevelBVH::get_closest_intersection over a ray batch on the reference's
// ThreadPool, dispatched as 4096-ray tasks round-robin like Util::Tiler.
// Returns wall seconds.
double ref_trace_timed(const void* p, const po_ray* rays, uint32_t n, po_hit* hits, int nthreads)
{
    const auto* s = static_cast<const RefScene*>(p);
    ThreadPool pool(nthreads > 0 ? (uint32_t)nthreads : std::thread::hardware_concurrency());
    const uint32_t chunk = 4096;
    auto t0 = std::chrono::steady_clock::now();
    std::vector<std::future<bool>> handles;
    auto task = [&](uint32_t lo, uint32_t hi) -> bool {
        for (uint32_t i = lo; i < hi; ++i) {
            Core::Ray ray = to_ray(rays[i]);
            InterpolatedVertex v{};
            if (s->tlas.get_closest_intersection(ray, &v)) {
                hits[i].inst = s->instance_of.at(v.m_bsrdf);
                hits[i].prim = prim_of(*s, hits[i].inst, v);
                hits[i].t = glm::length(v.mPosition - ray.mOrigin);
                hits[i].u = v.mUV.x; hits[i].v = v.mUV.y;
            } else {
                hits[i].inst = hits[i].prim = 0xffffffffu;
                hits[i].t = INFINITY; hits[i].u = hits[i].v = 0.0f;
            }
        }
        return true;
    };
    for (uint32_t lo = 0; lo < n; lo += chunk) handles.push_back(pool.add_task(task, lo, std::min(n, lo + chunk)));
    for (auto& h : handles) h.wait();
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

uint32_t ref_blas_node_count(const void* p, uint32_t mesh)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = (*static_cast<LowerLevelMeshBVH*>(s->blas[mesh].get())).*robbed(BlasTag{});
    return (uint32_t)((*bvh).*robbed(BNodesTag{})).size();
}
uint32_t ref_blas_root(const void* p, uint32_t mesh)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = (*static_cast<LowerLevelMeshBVH*>(s->blas[mesh].get())).*robbed(BlasTag{});
    return (*bvh).*robbed(BRootTag{});
}
void ref_blas_nodes(const void* p, uint32_t mesh, float* boxes, uint32_t* links, uint32_t* values)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = (*static_cast<LowerLevelMeshBVH*>(s->blas[mesh].get())).*robbed(BlasTag{});
    dump_nodes(bvh, 0, boxes, links, values, nullptr);
}
uint32_t ref_tlas_node_count(const void* p)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = s->tlas.*robbed(TlasTag{});
    return (uint32_t)((*bvh).*robbed(TNodesTag{})).size();
}
uint32_t ref_tlas_root(const void* p)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = s->tlas.*robbed(TlasTag{});
    return (*bvh).*robbed(TRootTag{});
}
void ref_tlas_nodes(const void* p, float* boxes, uint32_t* links, uint32_t* values)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto* bvh = s->tlas.*robbed(TlasTag{});
    const auto& entries = s->tlas.*robbed(EntriesTag{});
    dump_nodes(bvh, 0, boxes, links, values, &entries);
}
void ref_instance_inverse(const void* p, uint32_t inst, float* out)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto& entries = s->tlas.*robbed(EntriesTag{});
    std::memcpy(out, &entries[inst].mInverseTransform[0][0], sizeof(float) * 16);
}
// LowerLevelMeshBVH light sampling data: triangle weights and alias buckets.
uint32_t ref_light_table(const void* p, uint32_t mesh, float* areas, float* bucket_weight, uint32_t* bucket_alias)
{
    const auto* s = static_cast<const RefScene*>(p);
    const auto& area = (*static_cast<LowerLevelMeshBVH*>(s->blas[mesh].get())).*robbed(AreaTag{});
    const auto& table = (*static_cast<LowerLevelMeshBVH*>(s->blas[mesh].get())).*robbed(AliasTag{});
    const auto& buckets = table.*robbed(BucketsTag{});
    for (size_t i = 0; i < area.size(); ++i) {
        if (areas) areas[i] = area[i];
        if (bucket_weight) bucket_weight[i] = buckets[i].m_weight;
        if (bucket_alias) bucket_alias[i] = buckets[i].m_alias_index;
    }
    return (uint32_t)area.size();
}

void ref_mat4_inverse(const float* m, float* out)
{
    const glm::mat4 r = glm::inverse(to_mat4(m));
    std::memcpy(out, &r[0][0], sizeof(float) * 16);
}

void ref_generate_ray(const po_camera* c, float xi_x, float xi_y, uint32_t px, uint32_t py, po_ray* out)
{
    const Core::Ray r = to_camera(c).generate_ray(glm::vec2(xi_x, xi_y), glm::uvec2(px, py));
    out->org[0] = r.mOrigin.x; out->org[1] = r.mOrigin.y; out->org[2] = r.mOrigin.z; out->org[3] = r.mOrigin.w;
    out->dir[0] = r.mDirection.x; out->dir[1] = r.mDirection.y; out->dir[2] = r.mDirection.z; out->dir[3] = r.mLenght;
}

void ref_view_matrix(const po_camera* c, float* out)
{
    const glm::mat4 v = to_camera(c).getViewMatrix();
    std::memcpy(out, &v[0][0], sizeof(float) * 16);
}

// Random streams: n successive draws from a freshly seeded generator.
void ref_xorshift(uint32_t seed, uint32_t n, uint32_t* out)
{
    Core::Rand::xorshift_random r(seed);
    for (uint32_t i = 0; i < n; ++i) out[i] = r.next();
}
void ref_hammersley(uint32_t seed, uint32_t n, float* out)
{
    Core::Rand::Hammersley_Generator g(seed);
    for (uint32_t i = 0; i < n; ++i) {
        const glm::vec2 x = g.next();
        out[2 * i] = x.x; out[2 * i + 1] = x.y;
    }
}
float ref_radical_inverse(uint32_t bits) { return Core::Rand::radical_inverse_VdC(bits); }
void ref_uniform_sample_triangle(const float* xi, float* out)
{
    const glm::vec2 r = Core::Rand::uniform_sample_triangle(glm::vec2(xi[0], xi[1]));
    out[0] = r.x; out[1] = r.y;
}
void ref_mt_uniform(uint64_t seed, uint32_t n, float* out)
{
    std::mt19937_64 g{seed};
    std::uniform_real_distribution<float> d(0.0f, 1.0f);
    for (uint32_t i = 0; i < n; ++i) out[i] = d(g);
}

void ref_tangent_frame(const float* V, const float* N, float* out)
{
    const glm::mat3 m = Core::TangentSpace::construct_world_to_tangent_transform(glm::vec3(V[0], V[1], V[2]),
                                                                                  glm::vec3(N[0], N[1], N[2]));
    std::memcpy(out, &m[0][0], sizeof(float) * 9);
}
void ref_cos_sample(const float* xi, float* H)
{
    Render::Cos_Weighted_Hemisphere_Distribution d;
    const glm::vec3 h = d.sample(glm::vec2(xi[0], xi[1]), glm::vec3(0, 0, 1), 0.0f);
    H[0] = h.x; H[1] = h.y; H[2] = h.z;
}
float ref_cos_pdf(const float* H)
{
    Render::Cos_Weighted_Hemisphere_Distribution d;
    return d.pdf(glm::vec3(0, 0, 1), glm::vec3(H[0], H[1], H[2]), 0.0f);
}
void ref_beckmann_sample(const float* xi, const float* V, float R, float* H)
{
    Render::Beckmann_All_Microfacet_Distribution d;
    const glm::vec3 h = d.sample(glm::vec2(xi[0], xi[1]), glm::vec3(V[0], V[1], V[2]), R);
    H[0] = h.x; H[1] = h.y; H[2] = h.z;
}
float ref_beckmann_pdf(const float* H, float R)
{
    Render::Beckmann_All_Microfacet_Distribution d;
    return d.pdf(glm::vec3(0, 0, 1), glm::vec3(H[0], H[1], H[2]), R);
}

float ref_bsdf_pdf(int kind, const float* wo, const float* H, float roughness, float reflectance)
{
    RefScene s;
    po_material m{};
    std::unique_ptr<Core::Material> mat = std::make_unique<FixedMaterial>(m);
    s.materials.add_material(mat);
    auto b = make_bsrdf(s, (uint32_t)kind, 0);
    return b->pdf(glm::vec3(wo[0], wo[1], wo[2]), glm::vec3(H[0], H[1], H[2]), roughness, reflectance);
}

// BSRDF::sample with a Hammersley_Generator seeded by `seed`.
void ref_bsdf_sample(int kind, const po_material* material, const float* V, const float* N, uint32_t seed,
                     float* L, float* P, float* energy)
{
    RefScene s;
    std::unique_ptr<Core::Material> mat = std::make_unique<FixedMaterial>(*material);
    s.materials.add_material(mat);
    auto b = make_bsrdf(s, (uint32_t)kind, 0);
    Core::Rand::Hammersley_Generator g(seed);
    InterpolatedVertex frag{};
    frag.mNormal = glm::vec3(N[0], N[1], N[2]);
    Core::Ray ray{};
    ray.mDirection = -glm::vec3(V[0], V[1], V[2]);
    const Render::Sample smp = b->sample(g, frag, ray);
    L[0] = smp.L.x; L[1] = smp.L.y; L[2] = smp.L.z;
    *P = smp.P;
    energy[0] = smp.energy.x; energy[1] = smp.energy.y; energy[2] = smp.energy.z;
}

// The five lines of direct_lighting_pdf (Render/Integrators.cpp:13-22, in an
// anonymous namespace there), written against the reference's own routines.
float ref_direct_lighting_pdf(int kind, const po_material* material, const float* N, const float* wi, const float* wo)
{
    RefScene s;
    std::unique_ptr<Core::Material> mat = std::make_unique<FixedMaterial>(*material);
    s.materials.add_material(mat);
    auto b = make_bsrdf(s, (uint32_t)kind, 0);
    const Core::EvaluatedMaterial e = s.materials.evaluate_material(0, glm::vec2(0.0f));
    const glm::vec3 n(N[0], N[1], N[2]), vi(wi[0], wi[1], wi[2]), vo(wo[0], wo[1], wo[2]);
    const glm::mat3x3 tt = Core::TangentSpace::construct_world_to_tangent_transform(vi, n);
    const glm::vec3 two = tt * vo;
    glm::vec3 H = glm::normalize(vi + vo);
    H = tt * H;
    return b->pdf(two, H, e.roughness, e.get_reflectance());
}

// Monte_Carlo_Integrator::integrate_ray, nsamples successive samples of one integrator.
void ref_integrate(const void* p, const po_camera* c, uint32_t px, uint32_t py, uint32_t max_depth,
                   uint64_t seed, uint32_t nsamples, float* out)
{
    auto* s = const_cast<RefScene*>(static_cast<const RefScene*>(p));
    const Scene::Camera cam = to_camera(c);
    Render::Monte_Carlo_Integrator it(s->tlas, s->materials, s->lights, s->sun, seed);
    for (uint32_t i = 0; i < nsamples; ++i) {
        const glm::vec3 r = it.integrate_ray(cam, glm::uvec2(px, py), max_depth);
        out[3 * i] = r.x; out[3 * i + 1] = r.y; out[3 * i + 2] = r.z;
    }
}

// The per-pixel body of Scene::render_scene_to_memory (Core/Scene.cpp:164-198)
// over a list of pixels, each with its own integrator seed.  `nthreads`
// workers of the reference ThreadPool take 4096-pixel tasks; returns seconds.
double ref_render_pixels(const void* p, const po_camera* c, uint32_t max_depth, uint32_t max_samples,
                         float max_variance, const uint32_t* pixel_index, const uint64_t* seeds,
                         uint32_t npixels, float* pixels, uint32_t* counts, float* variance, int nthreads)
{
    auto* s = const_cast<RefScene*>(static_cast<const RefScene*>(p));
    const Scene::Camera cam = to_camera(c);
    const uint32_t W = c->resolution[0];
    glm::vec3* P = reinterpret_cast<glm::vec3*>(pixels);
    glm::vec3* V = reinterpret_cast<glm::vec3*>(variance);
    auto body = [&](uint32_t lo, uint32_t hi) -> bool {
        for (uint32_t k = lo; k < hi; ++k) {
            const uint32_t flat = pixel_index[k];
            if (counts[flat] >= max_samples) continue;
            const glm::uvec2 pix(flat % W, flat / W);
            Render::Monte_Carlo_Integrator integrator(s->tlas, s->materials, s->lights, s->sun, seeds[k]);
            for (uint32_t i = 0; i < max_samples; ++i) {
                uint32_t prev = counts[flat];
                glm::vec3 x = integrator.integrate_ray(cam, pix, max_depth);
                if (prev < 1) {
                    counts[flat] = 1;
                    V[flat] = glm::vec4(0, 0, 0, 0);
                } else {
                    const glm::vec3& pp = P[flat];
                    const glm::vec3& pv = V[flat];
                    const glm::vec3 np = pp + ((x - pp) * (1.0f / static_cast<float>(prev)));
                    V[flat] = ((pv * prev) + ((x - pp) * (x - np))) / (prev + 1);
                    counts[flat] = prev + 1;
                    x = np;
                }
                P[flat] = x;
                if (prev > 4 && glm::all(glm::lessThanEqual(V[flat], glm::vec3(max_variance)))) break;
            }
        }
        return true;
    };
    auto t0 = std::chrono::steady_clock::now();
    {
        ThreadPool pool(nthreads > 0 ? (uint32_t)nthreads : std::thread::hardware_concurrency());
        std::vector<std::future<bool>> handles;
        for (uint32_t lo = 0; lo < npixels; lo += 4096)
            handles.push_back(pool.add_task(body, lo, std::min(npixels, lo + 4096)));
        for (auto& h : handles) h.wait();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// A converged judge render: `spp` samples of the reference's own
// Monte_Carlo_Integrator::integrate_ray (Render/Integrators.cpp:130-154) per listed
// pixel, summed in double precision.  Writes per pixel and channel the plain mean
// of all samples and their unbiased sample variance (not the running mean of
// Scene.cpp:185-191, which drops the first sample).
double ref_render_mean64(const void* p, const po_camera* c, uint32_t max_depth, uint32_t spp,
                         const uint32_t* pixel_index, const uint64_t* seeds, uint32_t npixels, double* mean,
                         double* var, int nthreads)
{
    auto* s = const_cast<RefScene*>(static_cast<const RefScene*>(p));
    const Scene::Camera cam = to_camera(c);
    const uint32_t W = c->resolution[0];
    auto body = [&](uint32_t lo, uint32_t hi) -> bool {
        for (uint32_t k = lo; k < hi; ++k) {
            const uint32_t flat = pixel_index[k];
            const glm::uvec2 pix(flat % W, flat / W);
            Render::Monte_Carlo_Integrator integrator(s->tlas, s->materials, s->lights, s->sun, seeds[k]);
            double sum[3] = {0.0, 0.0, 0.0}, sq[3] = {0.0, 0.0, 0.0};
            for (uint32_t i = 0; i < spp; ++i) {
                const glm::vec3 x = integrator.integrate_ray(cam, pix, max_depth);
                for (int a = 0; a < 3; ++a) {
                    sum[a] += (double)x[a];
                    sq[a] += (double)x[a] * (double)x[a];
                }
            }
            for (int a = 0; a < 3; ++a) {
                const double m = sum[a] / spp;
                mean[3 * k + a] = m;
                var[3 * k + a] = spp > 1 ? (sq[a] - spp * m * m) / (spp - 1) : 0.0;
            }
        }
        return true;
    };
    auto t0 = std::chrono::steady_clock::now();
    {
        ThreadPool pool(nthreads > 0 ? (uint32_t)nthreads : std::thread::hardware_concurrency());
        std::vector<std::future<bool>> handles;
        for (uint32_t lo = 0; lo < npixels; lo += 16)
            handles.push_back(pool.add_task(body, lo, std::min(npixels, lo + 16)));
        for (auto& h : handles) h.wait();
    }
    auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

// Scene::generate_denoiser_inputs (Core/Scene.cpp:248-294), private there; the
// per-pixel body is written against the reference's public routines.
void ref_denoiser_inputs(const void* p, const po_camera* c, uint32_t W, uint32_t H, float* normals,
                         float* positions, float* diffuse)
{
    const auto* s = static_cast<const RefScene*>(p);
    const Scene::Camera cam = to_camera(c);
    for (uint32_t x = 0; x < W; ++x)
        for (uint32_t y = 0; y < H; ++y) {
            const uint32_t flat = y * W + x;
            Core::Ray ray = cam.generate_ray(glm::vec2(0.0f, 0.0f), glm::uvec2(x, y));
            InterpolatedVertex frag{};
            glm::vec3 n, pos, d;
            if (s->tlas.get_closest_intersection(ray, &frag)) {
                n = frag.mNormal;
                pos = cam.getViewMatrix() * frag.mPosition;
                d = s->materials.evaluate_material(frag.m_bsrdf->get_material_id(), frag.mUV).diffuse;
            } else {
                n = -ray.mDirection;
                pos = ray.mDirection * ray.mLenght;
                d = s->sun.m_sky_box->sample4(ray.mDirection);
            }
            std::memcpy(normals + 3 * flat, &n[0], 12);
            std::memcpy(positions + 3 * flat, &pos[0], 12);
            std::memcpy(diffuse + 3 * flat, &d[0], 12);
        }
}

// Util::atrous_denoise on a one-worker pool; returns seconds.
double ref_atrous(const float* pixels, const float* normals, const float* positions, const float* diffuse,
                  uint32_t W, uint32_t H, float* out, int nthreads)
{
    ThreadPool pool(nthreads > 0 ? (uint32_t)nthreads : 1u);
    Core::Rand::xorshift_random rng(1234u);
    Util::Tiler tiler(pool, rng, glm::uvec2(W, H), glm::uvec2(64, 64));
    auto t0 = std::chrono::steady_clock::now();
    glm::vec3* r = Util::atrous_denoise(reinterpret_cast<const glm::vec3*>(pixels),
                                        reinterpret_cast<const glm::vec3*>(normals),
                                        reinterpret_cast<const glm::vec3*>(positions),
                                        reinterpret_cast<const glm::vec3*>(diffuse), tiler);
    auto t1 = std::chrono::steady_clock::now();
    std::memcpy(out, r, sizeof(float) * 3 * (size_t)W * H);
    delete[] r;
    return std::chrono::duration<double>(t1 - t0).count();
}

// Util::reinhard_tone_mapping in place, on a one-worker pool.
void ref_reinhard(float* pixels, uint32_t W, uint32_t H)
{
    ThreadPool pool(1u);
    Core::Rand::xorshift_random rng(99u);
    Util::Tiler tiler(pool, rng, glm::uvec2(W, H), glm::uvec2(64, 64));
    Util::reinhard_tone_mapping(reinterpret_cast<glm::vec3*>(pixels), glm::uvec2(W, H), tiler);
}

// The output step of Scene::render_scene_to_file (Core/Scene.cpp:238-246) on a
// copy of the pixels: std::reverse, then stbi_write_hdr to `path`.
int ref_write_hdr(const float* pixels, uint32_t W, uint32_t H, const char* path)
{
    std::vector<glm::vec3> px(reinterpret_cast<const glm::vec3*>(pixels),
                              reinterpret_cast<const glm::vec3*>(pixels) + (size_t)W * H);
    std::reverse(px.begin(), px.end());
    return stbi_write_hdr(path, (int)W, (int)H, 3, reinterpret_cast<const float*>(px.data()));
}

} // extern "C"
