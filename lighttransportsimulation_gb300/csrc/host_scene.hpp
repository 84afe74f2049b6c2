// Host-side scene model: what the reference's loader builds on the device with `new`
// (core/SceneLoader.cuh:195-360, core/SceneLoader_kernels.cu:8-111), held here as flat
// tables that are uploaded to the GPU as structure-of-arrays.
#pragma once

#include <cstdint>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "image_io.hpp"

namespace lts {

// Allocator whose resize leaves new elements uninitialised (default-initialised) instead of
// zeroing them: the loader sizes each table once and fills every element in parallel, so a
// zeroing pass would only touch every page once more, on one thread.
template <class T>
struct NoInitAlloc : std::allocator<T> {
    using value_type = T;
    template <class U>
    struct rebind {
        using other = NoInitAlloc<U>;
    };
    NoInitAlloc() = default;
    template <class U>
    NoInitAlloc(const NoInitAlloc<U>&) noexcept {}
    template <class U>
    void construct(U* q) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new (static_cast<void*>(q)) U;
    }
    template <class U, class... A>
    void construct(U* q, A&&... a) {
        ::new (static_cast<void*>(q)) U(std::forward<A>(a)...);
    }
};
template <class T>
using HostVec = std::vector<T, NoInitAlloc<T>>;

enum TexKind : int32_t { TEX_CONSTANT = 0, TEX_FBM = 1, TEX_WRINKLED = 2, TEX_MARBLE = 3, TEX_WINDY = 4, TEX_IMAGE = 5 };
enum MatKind : int32_t {
    MAT_NONE = 0,   // 'M' in the reference: parsed, no material constructed -> no BSDF
    MAT_MATTE = 1,  // 'L' MatteMaterial (Material.cuh:31-55)
    MAT_GLASS = 2,  // 'G' GlassMaterial (Material.cuh:57-76)
    MAT_MIRROR = 3, // 'R' MirrorMaterial (Material.cuh:78-95)
    MAT_METAL = 4   // 'C' (grammar extension) MetalMaterial with alpha given directly (Material.cuh:97-130)
};
enum LightKind : int32_t { LIGHT_AREA = 0, LIGHT_INFINITE = 1, LIGHT_POINT = 2 };

struct HostTexture {
    int32_t kind = TEX_CONSTANT;
    float v[4] = {0, 0, 0, 0};  // constant rgb | octaves, omega | octaves, omega, scale, variation | image
};

struct HostMaterial {
    int32_t kind = MAT_NONE;
    HostTexture tex[2];  // matte Kd | glass R, T | mirror R | metal k, eta
    float extra = 0;     // matte sigma (degrees) | glass eta | metal alpha
    float on_a = 0, on_b = 0;  // Oren-Nayar A, B (models/Microfacet.cuh:18-25) for sigma != 0
};

struct HostLight {
    int32_t kind = LIGHT_AREA;
    int32_t prim = -1;          // area light: primitive index in scene order
    float L[3] = {0, 0, 0};     // Lemit / Lmap / I
    float p[3] = {0, 0, 0};     // point light position; infinite light world center
    float radius = 0;           // infinite light world radius
    float area = 0;             // area light triangle area
};

// An instanced mesh entry (the loader's `instances` grammar extension): mesh entry `mesh`
// places its file's triangles at p * s + t (before the subject transform, for subject meshes).
// Entries with the same mesh file share prototype `proto`, whose object-space triangles are
// HostScene::proto_soup[proto].
constexpr int kMaxSceneInstances = 32;  // instances one scene may hold (bits of a traversal mask)
struct HostInstance {
    int32_t mesh = 0, proto = 0;
    float t[3] = {0, 0, 0};
    float s = 1;
};

struct HostScene {
    int32_t width = 0, height = 0;
    // Camera (rendering/Camera.cu:9-43): o, right, up, llc, u, v, w, lensRadius, focalDist.
    float cam[23] = {0};
    // Gaussian filter table (rendering/Filter.cuh:32-50,82-99), 16 x 16, radius 1, alpha 1.
    float filter[256] = {0};

    // Vertex pools (world space) and per-triangle corner indices into them.
    HostVec<float> p;       // 3 per vertex
    HostVec<float> n;       // 3 per normal
    HostVec<float> uv;      // 2 per uv
    HostVec<int32_t> tri_p;   // 3 per triangle
    HostVec<int32_t> tri_n;   // 3 per triangle, -1 when the mesh has no normals
    HostVec<int32_t> tri_uv;  // 3 per triangle, -1 when the mesh has no uvs
    HostVec<int32_t> tri_mesh;

    std::vector<int32_t> mesh_first_tri, mesh_tri_count;
    int32_t subject_meshes = 0;
    int32_t area_light_meshes = 0;
    bool has_infinite = false;

    std::vector<HostMaterial> materials;  // one per mesh (material index == mesh index)
    HostVec<int32_t> prim_light;          // per triangle: light index or -1
    std::vector<HostLight> lights;        // sampling order of the reference's light array
    std::vector<float> light_func, light_cdf;  // Distribution1D over power().y()
    float light_func_int = 0;                  // Distribution1D::funcInt (before normalising)

    // Instanced mesh entries and their prototypes' object-space triangles (9 floats each, in
    // the mesh file's order); empty when the scene has no `instances` record.
    std::vector<HostInstance> instances;
    std::vector<std::vector<float>> proto_soup;

    // Image textures in the reference's image order (subject images first), each with its mip
    // pyramid (the fixed mode of ImageTexture / Mipmap).
    std::vector<HostImage> images;

    int32_t triangles() const { return (int32_t)tri_mesh.size(); }
    int32_t max_mesh_triangles() const;
    // World-space positions of every triangle, 9 floats each, in scene order.
    void triangle_soup(std::vector<float>& out) const;
};

struct AppParams {
    int32_t width = 0, height = 0, spp = 0, max_bounce = 0, rr_start = 0, format = 0;
    std::string output, scene, subject;
};

// All return "" on success, else an error message; *code receives an LTS_ERR_* value.
std::string read_app_params(const std::string& path, AppParams* out, int* code);
// core/FileIO.cuh:73-164: mesh_name.obj -> mesh_name.bin in the reference's binary layout.
std::string obj_to_bin(const std::string& mesh_name, int* code);
std::string load_scene(const std::string& root, const std::string& scene, const std::string& subject,
                       int32_t width, int32_t height, HostScene* out, int* code);

// Reference float helpers shared by loader code paths (host, no FMA contraction).
float quake_rsqrt(float f);

// The reference camera (rendering/Camera.cu:9-43, aperture 0) from a camera record
// cf = from(3), at(3), up(3), vfov in degrees, focus distance: cam[23] as HostScene::cam.
void build_camera(const float cf[11], int width, int height, float cam[23]);

}  // namespace lts
