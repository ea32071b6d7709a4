// eref_harness.cpp -- times the reference's CPU renderer on a scene file
// (TEST INFRASTRUCTURE ONLY: the CPU baseline of bench.py).
//
//   eref_harness SCENE FRAMES [STRIDE] [OUT]
//
// Reads the scene file written by oracle/ref/ref_io.py (the format
// ref_harness.cu reads), builds the reference's Mesh / SceneGraph /
// SceneManager / Camera / Texture objects and renders FRAMES frames with
// Elite::Renderer::Render (ERenderer.cpp:42-164, single-threaded as
// written).  STRIDE > 1 keeps every STRIDE-th triangle of each list mesh, a
// bounded sample of the frame's work.  The GPU shader's constant light is
// added as the scene's one directional light.  Prints one JSON line with the mean
// wall time per frame and the triangles rendered; OUT, if given, receives
// the back buffer (0x00RRGGBB words).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <unordered_map>
#include <vector>

#include <SDL.h>

#include "Camera.h"
#include "CullingMode.h"
#include "DirectionalLight.h"
#include "ERenderer.h"
#include "Mesh.h"
#include "SampleState.h"
#include "SceneGraph.h"
#include "SceneManager.h"
#include "Texture.h"
#include "Textures.h"
#include "VisualisationState.h"

void eref_set_window_size(int w, int h);
void eref_register_image(const char* name, const void* rgba8, int w, int h);

namespace {

std::unordered_map<const Mesh*, Textures> g_textures;

struct Reader {
    FILE* f;
    template <typename T> T get() {
        T v;
        if (fread(&v, sizeof v, 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); }
        return v;
    }
    void bytes(void* dst, size_t n) {
        if (n && fread(dst, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
    }
};

// A Camera whose look-at and projection matrices are the scene file's.
class FileCamera : public Camera {
public:
    FileCamera(const FPoint3& pos, const FMatrix4& view, const FMatrix4& proj) : Camera(pos, 60.f) {
        m_LookAtMatrix = Inverse(view);
        m_ProjectionMatrix = proj;
    }
};

}  // namespace

// The textures of a mesh (patch E1 of build_ref.py routes ERenderer here).
const Textures& ErefTexturesOf(const Mesh* pMesh) {
    static const Textures none{};
    auto it = g_textures.find(pMesh);
    return it == g_textures.end() ? none : it->second;
}

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s SCENE FRAMES [STRIDE] [OUT]\n", argv[0]);
        return 2;
    }
    const int frames = atoi(argv[2]);
    const uint32_t stride = argc > 3 ? (uint32_t)atoi(argv[3]) : 1u;
    FILE* fin = fopen(argv[1], "rb");
    if (!fin) { perror("scene"); return 2; }
    Reader rd{fin};
    if (rd.get<uint32_t>() != 0x53524247u) { fprintf(stderr, "bad magic\n"); return 2; }
    const uint32_t W = rd.get<uint32_t>(), H = rd.get<uint32_t>();
    for (int k = 0; k < 5; ++k) rd.get<uint32_t>();   // bins and queue size: the CPU renderer has none
    const CullingMode cm = (CullingMode)rd.get<uint32_t>();
    const SampleState ss = (SampleState)rd.get<uint32_t>();
    const VisualisationState vs = (VisualisationState)rd.get<uint32_t>();
    float pos[3], fwd[3];
    FMatrix4 view, proj;
    rd.bytes(pos, 12);
    rd.bytes(fwd, 12);
    rd.bytes(&view, 64);
    rd.bytes(&proj, 64);

    const uint32_t ntex = rd.get<uint32_t>();
    std::vector<Texture*> textures(ntex);
    for (uint32_t t = 0; t < ntex; ++t) {
        const uint32_t tw = rd.get<uint32_t>(), th = rd.get<uint32_t>();
        std::vector<uint32_t> px((size_t)tw * th);
        rd.bytes(px.data(), px.size() * 4u);
        const std::string name = "texture" + std::to_string(t);
        eref_register_image(name.c_str(), px.data(), (int)tw, (int)th);
        textures[t] = new Texture(name.c_str());
    }

    SceneGraph* sg = new SceneGraph();
    uint64_t tris = 0;
    const uint32_t nmesh = rd.get<uint32_t>();
    for (uint32_t m = 0; m < nmesh; ++m) {
        const uint32_t nv = rd.get<uint32_t>();
        IVertex* verts = new IVertex[nv];
        rd.bytes(verts, (size_t)nv * sizeof(IVertex));
        const uint32_t ni = rd.get<uint32_t>();
        std::vector<uint32_t> idx(ni);
        rd.bytes(idx.data(), (size_t)ni * 4u);
        const uint32_t topo = rd.get<uint32_t>();
        FMatrix4 world;
        rd.bytes(&world, 64);
        int32_t tex[4];
        rd.bytes(tex, 16);
        if (topo == 0 && stride > 1) {   // a bounded sample: every stride-th triangle
            std::vector<uint32_t> kept;
            for (uint32_t t = 0; 3u * t + 2u < ni; t += stride) kept.insert(kept.end(), &idx[3u * t], &idx[3u * t] + 3);
            idx.swap(kept);
        }
        unsigned int* ib = new unsigned int[idx.size()];
        std::memcpy(ib, idx.data(), idx.size() * 4u);
        Mesh* mesh = new Mesh{verts, nv, 56, 0, ib, (unsigned int)idx.size(), (PrimitiveTopology)topo};
        mesh->GetWorld() = world;
        Textures tx{};
        Texture** slots[4] = {&tx.pDiff, &tx.pNorm, &tx.pSpec, &tx.pGloss};
        for (int k = 0; k < 4; ++k)
            if (tex[k] >= 0 && (uint32_t)tex[k] < ntex) *slots[k] = textures[tex[k]];
        g_textures[mesh] = tx;
        sg->AddMesh(mesh);
        tris += topo == 0 ? idx.size() / 3u : (idx.size() >= 2u ? idx.size() - 2u : 0u);
    }
    fclose(fin);
    // the GPU shader's constant light (CUDAROPs.cu:417-420) as a scene light,
    // which is what the CPU renderer shades with
    sg->AddLight(new DirectionalLight(RGBColor{1.f, 1.f, 1.f}, 7.f, FVector3{0.577f, -0.577f, -0.577f}));

    SceneManager sm;
    sm.AddSceneGraph(sg);
    sm.m_CullingMode = cm;
    sm.m_SampleState = ss;
    sm.m_Visualisation = vs;
    FileCamera camera(FPoint3{pos[0], pos[1], pos[2]}, view, proj);

    eref_set_window_size((int)W, (int)H);
    Elite::Renderer renderer(nullptr);
    renderer.SetCamera(&camera);
    renderer.Render(sm);   // warm-up
    const auto t0 = std::chrono::steady_clock::now();
    for (int f = 0; f < frames; ++f) renderer.Render(sm);
    const auto t1 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / (frames > 0 ? frames : 1);
    printf("{\"ms_per_frame\": %.4f, \"triangles\": %llu, \"frames\": %d, \"stride\": %u, \"threads\": 1}\n", ms,
           (unsigned long long)tris, frames, stride);
    if (argc > 4) {
        SDL_Surface* back = renderer.m_pBackBuffer;
        FILE* fo = fopen(argv[4], "wb");
        if (fo) {
            fwrite(back->pixels, 4, (size_t)W * H, fo);
            fclose(fo);
        }
    }
    return 0;
}
