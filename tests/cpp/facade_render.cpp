// facade_render.cpp -- renders a scene file through the C++ host API
// (include/gbr_cudarenderer.hpp) the way an application written against
// the reference's CUDARenderer would: fill a SceneGraph and a
// CUDATextureManager, LoadScene, SetupBins, Render, Present.
//
// usage: facade_render <scene.bin> <out.bin>
// scene.bin: the format written by oracle/ref/ref_io.py (IVertex meshes);
// out.bin: width, height (uint32) then the framebuffer words and depth.
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "gbr_cudarenderer.hpp"

namespace {
template <typename T>
T get(FILE* f) {
    T v;
    if (fread(&v, sizeof v, 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); }
    return v;
}
void bytes(FILE* f, void* dst, size_t n) {
    if (n && fread(dst, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
}
}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s scene.bin out.bin\n", argv[0]); return 2; }
    FILE* f = fopen(argv[1], "rb");
    if (!f) { perror("scene"); return 2; }
    if (get<uint32_t>(f) != 0x53524247u) { fprintf(stderr, "bad magic\n"); return 2; }
    const uint32_t W = get<uint32_t>(f), H = get<uint32_t>(f);
    const int nbx = (int)get<uint32_t>(f), nby = (int)get<uint32_t>(f);
    const int bw = (int)get<uint32_t>(f), bh = (int)get<uint32_t>(f);
    (void)get<uint32_t>(f);  // queue capacity of the reference: bins are exact-sized here
    gbr::SceneManager sm;
    sm.SetCullingMode((gbr::CullingMode)get<uint32_t>(f));
    sm.SetSampleState((gbr::SampleState)get<uint32_t>(f));
    sm.SetVisualisationState((gbr::VisualisationState)get<uint32_t>(f));
    gbr_camera cam{};
    bytes(f, cam.pos, 12);
    bytes(f, cam.fwd, 12);
    bytes(f, cam.view, 64);
    bytes(f, cam.proj, 64);

    gbr::CUDATextureManager tm;
    const uint32_t ntex = get<uint32_t>(f);
    for (uint32_t t = 0; t < ntex; ++t) {
        const uint32_t tw = get<uint32_t>(f), th = get<uint32_t>(f);
        std::vector<uint32_t> px((size_t)tw * th);
        bytes(f, px.data(), px.size() * 4u);
        tm.AddCUDATexture(std::move(px), tw, th);
    }
    gbr::SceneGraph sg;
    std::vector<gbr::Mesh> meshes;
    const uint32_t nmesh = get<uint32_t>(f);
    meshes.reserve(nmesh);
    for (uint32_t m = 0; m < nmesh; ++m) {
        std::vector<gbr::IVertex> v(get<uint32_t>(f));
        bytes(f, v.data(), v.size() * sizeof(gbr::IVertex));
        std::vector<uint32_t> ix(get<uint32_t>(f));
        bytes(f, ix.data(), ix.size() * 4u);
        const auto topo = (gbr::PrimitiveTopology)get<uint32_t>(f);
        meshes.emplace_back(std::move(v), std::move(ix), topo);
        bytes(f, meshes.back().GetWorld().m, 64);
        int32_t tex[4];
        bytes(f, tex, 16);
        meshes.back().SetTextureIds(tex[0], tex[1], tex[2], tex[3]);
    }
    fclose(f);
    for (auto& m : meshes) sg.AddMesh(&m);

    try {
        gbr::CUDARenderer renderer(W, H);
        renderer.SetupBins(gbr::IPoint2{nbx, nby}, gbr::IPoint2{bw, bh});
        renderer.LoadScene(&sg, tm);
        renderer.Render(sm, tm, cam);  // camera matrices from the scene file
        std::vector<uint32_t> colour((size_t)W * H);
        std::vector<float> depth((size_t)W * H);
        renderer.Present(colour.data(), depth.data());
        FILE* o = fopen(argv[2], "wb");
        if (!o) { perror("out"); return 2; }
        fwrite(&W, 4, 1, o);
        fwrite(&H, 4, 1, o);
        fwrite(colour.data(), 4, colour.size(), o);
        fwrite(depth.data(), 4, depth.size(), o);
        fclose(o);
        printf("rendered %ux%u: %u of %u triangles visible\n", W, H, renderer.GetTotalNumVisibleTriangles(),
               renderer.GetTotalNumTriangles());
    } catch (const gbr::Error& e) {
        fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
