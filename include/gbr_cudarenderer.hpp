// gbr_cudarenderer.hpp -- header-only C++ host API over include/gbr.h with
// the shape of the reference's CUDARenderer and its scene classes, so that
// code written against CustomCUDARasterizer/CUDARenderer.h switches by
// changing includes:
//
//   CUDARenderer        CUDARenderer.h:31-141 (headless: Present copies into
//                       caller memory instead of an SDL surface)
//   CUDATextureManager  CUDATextureManager.h:12-14 (ids stay stable on removal)
//   Mesh, SceneGraph    Mesh.h:17-20,38-39,50, SceneGraph.h
//   Camera              Camera.h:7-35 (position, FOV, aspect, near/far; the
//                       projection keeps data[3][3] = 1 as Camera.cpp:97-108)
//   SceneManager        the render-state getters of SceneManager.h:19-22
//
// Errors: methods throw gbr::Error carrying the gbr_status and message of the
// failing C call (the reference has no error channel; CheckErrorCuda prints
// only in debug builds, PCH.h:46-56).
#pragma once
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "gbr.h"

namespace gbr {

struct Error : std::runtime_error {
    gbr_status status;
    Error(gbr_status s, const std::string& what) : std::runtime_error(what), status(s) {}
};

inline void check(gbr_status s, const char* call) {
    if (s != GBR_OK) throw Error(s, std::string(call) + ": " + gbr_last_error_string());
}

enum class CullingMode { BackFace = GBR_CULL_BACKFACE, FrontFace = GBR_CULL_FRONTFACE, NoCulling = GBR_CULL_NONE };
enum class SampleState { Point = GBR_SAMPLE_POINT, Linear = GBR_SAMPLE_LINEAR };
enum class VisualisationState { PBR = GBR_VIS_PBR, Depth = GBR_VIS_DEPTH, Normal = GBR_VIS_NORMAL };
enum class PrimitiveTopology : unsigned char { TriangleList = 0, TriangleStrip = 1 };

struct IPoint2 { int x, y; };

// IVertex (Vertex.h:113-145), 56 bytes: position, uv, normal, tangent, colour.
struct IVertex {
    float p[3];
    float uv[2];
    float n[3];
    float tan[3];
    float c[3];
};
static_assert(sizeof(IVertex) == 56, "IVertex is 56 bytes");

// Column-major 4x4, element (r, c) at m[c * 4 + r] (Matrix.h:9-21).
struct FMatrix4 {
    float m[16];
    static FMatrix4 Identity() {
        FMatrix4 r{};
        r.m[0] = r.m[5] = r.m[10] = r.m[15] = 1.f;
        return r;
    }
};

class Mesh {
public:
    enum TextureID { Diffuse, Normal, Specular, Glossiness };
    Mesh(std::vector<IVertex> vertices, std::vector<uint32_t> indices, PrimitiveTopology topology)
        : m_Vertices(std::move(vertices)), m_Indices(std::move(indices)), m_Topology(topology),
          m_World(FMatrix4::Identity()) {}
    FMatrix4& GetWorld() { return m_World; }
    const FMatrix4& GetWorldConst() const { return m_World; }
    PrimitiveTopology GetTopology() const { return m_Topology; }
    const std::vector<IVertex>& GetVertexBuffer() const { return m_Vertices; }
    const std::vector<uint32_t>& GetIndexBuffer() const { return m_Indices; }
    const int* GetTextureIds() const { return m_TextureIds; }
    void SetTextureIds(int diff, int norm = -1, int spec = -1, int gloss = -1) {
        m_TextureIds[0] = diff; m_TextureIds[1] = norm; m_TextureIds[2] = spec; m_TextureIds[3] = gloss;
    }
    void SetTextureId(int id, TextureID slot = Diffuse) { m_TextureIds[slot] = id; }
    unsigned int GetTotalNumTriangles() const {
        return m_Topology == PrimitiveTopology::TriangleList ? (unsigned)(m_Indices.size() / 3)
                                                             : (unsigned)(m_Indices.size() >= 2 ? m_Indices.size() - 2 : 0);
    }

private:
    std::vector<IVertex> m_Vertices;
    std::vector<uint32_t> m_Indices;
    PrimitiveTopology m_Topology;
    FMatrix4 m_World;
    int m_TextureIds[4] = {-1, -1, -1, -1};
};

class SceneGraph {
public:
    void AddMesh(Mesh* pMesh) { m_pMeshes.push_back(pMesh); }
    const std::vector<Mesh*>& GetMeshes() const { return m_pMeshes; }

private:
    std::vector<Mesh*> m_pMeshes;
};

// Texture registry; textures are RGBA8 with byte0 = red (RGBRaw.h:34-38).
class CUDATextureManager {
public:
    struct Texture {
        std::vector<uint32_t> texels;
        unsigned int w = 0, h = 0;
    };
    int AddCUDATexture(std::vector<uint32_t> rgba8, unsigned int w, unsigned int h) {
        if (rgba8.size() != (size_t)w * h) throw Error(GBR_ERR_INVALID_ARG, "AddCUDATexture: size mismatch");
        m_Textures.push_back(Texture{std::move(rgba8), w, h});
        return (int)m_Textures.size() - 1;
    }
    const Texture* GetCUDATexture(int id) const {
        return id >= 0 && (size_t)id < m_Textures.size() && m_Textures[id].w ? &m_Textures[id] : nullptr;
    }
    void RemoveCUDATexture(int id) {
        if (id >= 0 && (size_t)id < m_Textures.size()) m_Textures[id] = Texture{};
    }
    size_t Size() const { return m_Textures.size(); }

private:
    std::vector<Texture> m_Textures;
};

class Camera {
public:
    explicit Camera(const float position[3], float fovDeg = 45.f) {
        for (int i = 0; i < 3; ++i) m_Position[i] = position[i];
        SetFov(fovDeg);
    }
    void SetFov(float degrees) {
        const float radians = degrees * (3.14159265358979323846f / 180.f);
        m_TanHalfFov = std::tan(radians / 2.f);
        Recalculate();
    }
    void SetAspectRatio(float width, float height) { m_Aspect = width / height; Recalculate(); }
    void SetNearFarValues(float nearZ, float farZ) { m_Near = nearZ; m_Far = farZ; Recalculate(); }
    // the camera state Render() reads (CUDARenderer.cu:215-219); an un-rotated
    // camera looks down -z with forward (0,0,1) and view = translation(-pos)
    gbr_camera State() const {
        gbr_camera c{};
        for (int i = 0; i < 3; ++i) c.pos[i] = m_Position[i];
        c.fwd[0] = 0.f; c.fwd[1] = 0.f; c.fwd[2] = 1.f;
        FMatrix4 v = FMatrix4::Identity();
        v.m[12] = -m_Position[0]; v.m[13] = -m_Position[1]; v.m[14] = -m_Position[2];
        std::memcpy(c.view, v.m, sizeof c.view);
        std::memcpy(c.proj, m_Proj.m, sizeof c.proj);
        return c;
    }

private:
    void Recalculate() {
        m_Proj = FMatrix4::Identity();
        const float A = m_Far / (m_Near - m_Far);
        const float B = (m_Far * m_Near) / (m_Near - m_Far);
        m_Proj.m[0] = 1.f / (m_Aspect * m_TanHalfFov);
        m_Proj.m[5] = 1.f / m_TanHalfFov;
        m_Proj.m[10] = A;
        m_Proj.m[11] = -1.f;
        m_Proj.m[14] = B;
    }
    float m_Position[3];
    float m_TanHalfFov = 1.f, m_Aspect = 1.f, m_Near = 0.1f, m_Far = 100.f;
    FMatrix4 m_Proj = FMatrix4::Identity();
};

class SceneManager {
public:
    VisualisationState GetVisualisationState() const { return m_Vis; }
    SampleState GetSampleState() const { return m_Sample; }
    CullingMode GetCullingMode() const { return m_Cull; }
    void SetVisualisationState(VisualisationState v) { m_Vis = v; }
    void SetSampleState(SampleState s) { m_Sample = s; }
    void SetCullingMode(CullingMode c) { m_Cull = c; }

private:
    // defaults of SceneManager.cpp:11-17
    VisualisationState m_Vis = VisualisationState::PBR;
    SampleState m_Sample = SampleState::Point;
    CullingMode m_Cull = CullingMode::BackFace;
};

class CUDARenderer final {
public:
    CUDARenderer(unsigned int width, unsigned int height, void* stream = nullptr) : m_W(width), m_H(height), m_Stream(stream) {
        check(gbr_create(width, height, &m_R), "gbr_create");
    }
    ~CUDARenderer() noexcept { gbr_destroy(m_R); }
    CUDARenderer(const CUDARenderer&) = delete;
    CUDARenderer& operator=(const CUDARenderer&) = delete;

    void SetupBins(const IPoint2& numBins, const IPoint2& binDim, unsigned int queueChunk = 256) {
        check(gbr_setup_bins(m_R, (uint32_t)numBins.x, (uint32_t)numBins.y, (uint32_t)binDim.x, (uint32_t)binDim.y,
                             queueChunk), "gbr_setup_bins");
    }

    void LoadScene(const SceneGraph* pSceneGraph, const CUDATextureManager& tm) {
        if (!pSceneGraph) throw Error(GBR_ERR_INVALID_ARG, "LoadScene: invalid scenegraph");
        check(gbr_scene_clear(m_R), "gbr_scene_clear");
        m_TexIds.assign(tm.Size(), -1);
        m_TotalNumTriangles = 0;
        for (const Mesh* pMesh : pSceneGraph->GetMeshes()) {
            int32_t ids[4];
            for (int k = 0; k < 4; ++k) ids[k] = DeviceTexture(tm, pMesh->GetTextureIds()[k]);
            const auto& v = pMesh->GetVertexBuffer();
            const auto& ix = pMesh->GetIndexBuffer();
            uint32_t mesh_id = 0;
            check(gbr_mesh_upload(m_R, v.data(), (uint32_t)v.size(), GBR_VERTEX_IVERTEX56, ix.data(),
                                  (uint32_t)ix.size(), (uint32_t)pMesh->GetTopology(), pMesh->GetWorldConst().m, ids,
                                  &mesh_id), "gbr_mesh_upload");
            m_TotalNumTriangles += pMesh->GetTotalNumTriangles();
        }
    }

    void Render(const SceneManager& sm, const CUDATextureManager& tm, const Camera* pCamera) {
        Render(sm, tm, pCamera->State());
    }

    // Render with explicit camera matrices (for cameras built elsewhere).
    void Render(const SceneManager& sm, const CUDATextureManager&, const gbr_camera& cam) {
        check(gbr_render(m_R, &cam, (uint32_t)sm.GetCullingMode(), (uint32_t)sm.GetSampleState(),
                         (uint32_t)sm.GetVisualisationState(), m_Stream), "gbr_render");
    }

    // Present without a window: the framebuffer words (bytes B, G, R, 0).
    void Present(uint32_t* pixels, float* depth = nullptr) {
        check(gbr_readback(m_R, pixels, depth, m_Stream), "gbr_readback");
    }

    void RenderAuto(const SceneManager& sm, const CUDATextureManager& tm, const Camera* pCamera, uint32_t* pixels) {
        Render(sm, tm, pCamera);
        Present(pixels);
    }

    unsigned int GetTotalNumVisibleTriangles() {
        gbr_stats st{};
        check(gbr_get_stats(m_R, &st, m_Stream), "gbr_get_stats");
        return (unsigned int)st.num_visible;
    }
    unsigned int GetTotalNumTriangles() const { return m_TotalNumTriangles; }
    gbr_renderer* Handle() const { return m_R; }

private:
    int DeviceTexture(const CUDATextureManager& tm, int id) {
        const CUDATextureManager::Texture* t = tm.GetCUDATexture(id);
        if (!t) return -1;
        if (m_TexIds[id] < 0) {
            int32_t dev_id = -1;
            check(gbr_texture_upload(m_R, t->texels.data(), t->w, t->h, &dev_id), "gbr_texture_upload");
            m_TexIds[id] = dev_id;
        }
        return m_TexIds[id];
    }

    gbr_renderer* m_R = nullptr;
    unsigned int m_W, m_H;
    void* m_Stream;
    unsigned int m_TotalNumTriangles = 0;
    std::vector<int> m_TexIds;
};

}  // namespace gbr
