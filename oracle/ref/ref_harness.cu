// ref_harness.cu -- drives the reference's own CUDARenderer on one scene and
// dumps what it produced (TEST INFRASTRUCTURE ONLY; built by build_ref.py
// against the staged, patched reference sources).
//
// usage: ref_harness <scene.bin> <out.bin> [--no-bins]
//
// The frame follows CUDARenderer::Render (CustomCUDARasterizer/
// CUDARenderer.cu:206-354) step by step through the reference's own
// launchers, with the camera matrices taken from the scene file instead of
// a Camera object, and with each mesh's world matrix set on its CUDAMesh
// verbatim.  After every TriangleBinner launch the bin queues are compacted
// on the device and copied out, so the dump holds the union over chunks of
// (bin, primitive id) pairs.  The output also holds the framebuffer and the
// interpolated z of every pixel's fragment (PixelShade::zInterpolated).
#include "CUDARenderer.cu"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <unordered_map>
#include <vector>

static_assert(sizeof(IVertex) == 56, "IVertex layout");
static_assert(sizeof(PixelShade) == 152, "PixelShade layout");

namespace {

struct Reader {
    FILE* f;
    template <typename T>
    T get() {
        T v;
        if (fread(&v, sizeof v, 1, f) != 1) { fprintf(stderr, "short read\n"); exit(2); }
        return v;
    }
    void bytes(void* dst, size_t n) {
        if (n && fread(dst, 1, n, f) != n) { fprintf(stderr, "short read\n"); exit(2); }
    }
};

// CUDATexture filled from memory in place of IMG_Load (CUDATexture.cpp:24-72)
class MemoryTexture : public CUDATexture {
public:
    bool CreateFromPixels(const uint32_t* px, unsigned int w, unsigned int h) {
        Destroy();
        unsigned int* dev = nullptr;
        size_t pitch = 0;
        if (cudaMallocPitch((void**)&dev, &pitch, w * 4u, h) != cudaSuccess) return false;
        if (cudaMemcpy2D(dev, pitch, px, w * 4u, w * 4u, h, cudaMemcpyHostToDevice) != cudaSuccess) return false;
        cudaResourceDesc resDesc{};
        resDesc.resType = cudaResourceTypePitch2D;
        resDesc.res.pitch2D.devPtr = dev;
        resDesc.res.pitch2D.desc.f = cudaChannelFormatKindUnsigned;
        resDesc.res.pitch2D.desc.x = 32;
        resDesc.res.pitch2D.width = w;
        resDesc.res.pitch2D.height = h;
        resDesc.res.pitch2D.pitchInBytes = pitch;
        cudaTextureDesc texDesc{};
        texDesc.normalizedCoords = true;
        texDesc.filterMode = cudaFilterModePoint;
        texDesc.readMode = cudaReadModeElementType;
        cudaTextureObject_t obj{};
        if (cudaCreateTextureObject(&obj, &resDesc, &texDesc, nullptr) != cudaSuccess) return false;
        m_Dev_pTex = obj;
        m_Width = w;
        m_Height = h;
        m_Dev_TextureData = dev;
        m_BytesPerPixel = 4;
        return true;
    }
};

// Compacts the occupied slots of the bin queues into (bin, queue entry) pairs.
__global__ void compact_queues(const unsigned int* sizes, const unsigned int* queues, unsigned int num_bins,
                               unsigned int cap, uint2* out, unsigned int* count) {
    const unsigned int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= num_bins * cap) return;
    const unsigned int b = i / cap, k = i % cap;
    if (k < sizes[b]) {
        const unsigned int pos = atomicAdd(count, 1u);
        out[pos] = make_uint2(b, queues[i]);
    }
}

struct TripleHash {
    size_t operator()(const std::tuple<unsigned, unsigned, unsigned>& t) const {
        return (size_t)std::get<0>(t) * 0x9E3779B97F4A7C15ull ^ (size_t)std::get<1>(t) * 0xC2B2AE3D27D4EB4Full ^
               (size_t)std::get<2>(t);
    }
};

}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) {
        fprintf(stderr, "usage: %s scene.bin out.bin [--no-bins]\n", argv[0]);
        return 2;
    }
    const bool want_bins = !(argc > 3 && strcmp(argv[3], "--no-bins") == 0);
    FILE* fin = fopen(argv[1], "rb");
    if (!fin) { perror("scene"); return 2; }
    Reader rd{fin};
    if (rd.get<uint32_t>() != 0x53524247u) { fprintf(stderr, "bad magic\n"); return 2; }
    const uint32_t W = rd.get<uint32_t>(), H = rd.get<uint32_t>();
    const uint32_t nbx = rd.get<uint32_t>(), nby = rd.get<uint32_t>();
    const uint32_t bw = rd.get<uint32_t>(), bh = rd.get<uint32_t>();
    const uint32_t qmax = rd.get<uint32_t>();
    const CullingMode cm = (CullingMode)rd.get<uint32_t>();
    const SampleState ss = (SampleState)rd.get<uint32_t>();
    const VisualisationState vs = (VisualisationState)rd.get<uint32_t>();
    FPoint3 camPos;
    FVector3 camFwd;
    FMatrix4 view, proj;
    rd.bytes(&camPos, 12);
    rd.bytes(&camFwd, 12);
    rd.bytes(&view, 64);
    rd.bytes(&proj, 64);

    SetDeviceCuda(0);
    WindowHelper wh;
    wh.Resolution.Width = W;
    wh.Resolution.Height = H;
    CUDARenderer renderer{wh};
    renderer.SetupBins(IPoint2{(int)nbx, (int)nby}, IPoint2{(int)bw, (int)bh}, qmax);

    CUDATextureManager tm;
    const uint32_t ntex = rd.get<uint32_t>();
    for (uint32_t t = 0; t < ntex; ++t) {
        const uint32_t tw = rd.get<uint32_t>(), th = rd.get<uint32_t>();
        std::vector<uint32_t> px((size_t)tw * th);
        rd.bytes(px.data(), px.size() * 4u);
        MemoryTexture* tex = new MemoryTexture();
        if (!tex->CreateFromPixels(px.data(), tw, th)) { fprintf(stderr, "texture upload failed\n"); return 3; }
        tm.AddCUDATexture(tex);
    }

    SceneGraph sg;
    const uint32_t nmesh = rd.get<uint32_t>();
    std::vector<FMatrix4> worlds(nmesh);
    std::vector<std::vector<uint32_t>> mesh_indices(nmesh);
    std::vector<uint32_t> mesh_topology(nmesh);
    std::vector<uint64_t> prim_base(nmesh);
    uint64_t total_tris = 0;
    for (uint32_t m = 0; m < nmesh; ++m) {
        const uint32_t nv = rd.get<uint32_t>();
        IVertex* verts = new IVertex[nv];
        rd.bytes(verts, (size_t)nv * sizeof(IVertex));
        const uint32_t ni = rd.get<uint32_t>();
        unsigned int* idx = new unsigned int[ni];
        rd.bytes(idx, (size_t)ni * 4u);
        mesh_indices[m].assign(idx, idx + ni);
        const uint32_t topo = rd.get<uint32_t>();
        mesh_topology[m] = topo;
        rd.bytes(&worlds[m], 64);
        int32_t tex[4];
        rd.bytes(tex, 16);
        Mesh* mesh = new Mesh{verts, nv, 56, 0, idx, ni, (PrimitiveTopology)topo};
        mesh->SetTextureIds(tex[0], tex[1], tex[2], tex[3]);
        sg.AddMesh(mesh);
        prim_base[m] = total_tris;
        total_tris += mesh->GetTotalNumTriangles();
    }
    fclose(fin);
    renderer.LoadScene(&sg, tm);
    for (uint32_t m = 0; m < nmesh; ++m) renderer.m_CUDAMeshes[m].pCUDAMesh->GetWorld() = worlds[m];

    const unsigned int num_bins = nbx * nby;
    uint2* d_pairs = nullptr;
    unsigned int* d_count = nullptr;
    cudaMalloc(&d_pairs, (size_t)num_bins * qmax * sizeof(uint2));
    cudaMalloc(&d_count, sizeof(unsigned int));
    std::vector<uint2> chunk_pairs;
    std::vector<std::pair<uint32_t, uint32_t>> bins_out;

    // EnterValidRenderingState (CUDARenderer.cu:373-381) without a surface
    renderer.Clear();
    // Render (CUDARenderer.cu:206-354)
    const FMatrix4 viewProjectionMatrix = proj * view;
    renderer.UpdateCameraDataAsync(camPos, camFwd);
    uint64_t total_visible = 0;
    for (uint32_t m = 0; m < nmesh; ++m) {
        CUDARenderer::SortedCUDAMesh& sm = renderer.m_CUDAMeshes[m];
        const CUDAMesh* pCudaMesh = sm.pCUDAMesh;
        const FMatrix4& worldMat = pCudaMesh->GetWorldConst();
        const FMatrix4 wvp = viewProjectionMatrix * worldMat;
        const FMatrix3& rot = pCudaMesh->GetRotationMatrix();
        renderer.UpdateWorldMatrixDataAsync(worldMat, wvp, rot);
        cudaDeviceSynchronize();
        renderer.VertexShader(pCudaMesh);
        cudaDeviceSynchronize();
        cudaMemset(renderer.m_Dev_NumVisibleTriangles, 0, sizeof(unsigned int));
        int binnerStatus = 0;
        cudaMemcpyToSymbol(dev_ConstMemory, &binnerStatus, sizeof(int), IsFinishedBinningIdx * 4);
        renderer.TriangleAssembler(pCudaMesh, camFwd, cm);
        cudaDeviceSynchronize();
        unsigned int nvis = 0;
        cudaMemcpy(&nvis, renderer.m_Dev_NumVisibleTriangles, 4, cudaMemcpyDeviceToHost);
        sm.NumVisibleTriangles = nvis;
        total_visible += nvis;
        // compacted triangle -> primitive id
        std::vector<TriangleIdx> tris(nvis);
        if (nvis) cudaMemcpy(tris.data(), pCudaMesh->GetDevTriangleBuffer(), nvis * sizeof(TriangleIdx), cudaMemcpyDeviceToHost);
        std::unordered_map<std::tuple<unsigned, unsigned, unsigned>, uint32_t, TripleHash> lut;
        const std::vector<uint32_t>& ix = mesh_indices[m];
        if (mesh_topology[m] == 0)
            for (uint32_t t = 0; t + 2 < ix.size() + 0 && 3 * t + 2 < ix.size(); ++t)
                lut.emplace(std::make_tuple(ix[3 * t], ix[3 * t + 1], ix[3 * t + 2]), t);
        std::vector<uint32_t> prim_of(nvis);
        for (uint32_t i = 0; i < nvis; ++i) {
            auto it = lut.find(std::make_tuple(tris[i].idx0, tris[i].idx1, tris[i].idx2));
            prim_of[i] = it == lut.end() ? 0xFFFFFFFFu : (uint32_t)(prim_base[m] + it->second);
        }
        const unsigned int queueMaxSize = renderer.m_BinQueues.GetQueueMaxSize();
        const unsigned int numLoops = (nvis + (queueMaxSize - 1)) / queueMaxSize;
        for (unsigned int i = 0; i < numLoops; ++i) {
            renderer.TriangleBinner(pCudaMesh, nvis, i * queueMaxSize);
            cudaDeviceSynchronize();
            if (want_bins) {
                cudaMemset(d_count, 0, 4);
                const unsigned int slots = num_bins * queueMaxSize;
                compact_queues<<<(slots + 255) / 256, 256>>>(renderer.m_BinQueues.GetDev_QueueSizes(),
                                                             renderer.m_BinQueues.GetDev_Queues(), num_bins,
                                                             queueMaxSize, d_pairs, d_count);
                unsigned int n = 0;
                cudaMemcpy(&n, d_count, 4, cudaMemcpyDeviceToHost);
                chunk_pairs.resize(n);
                if (n) cudaMemcpy(chunk_pairs.data(), d_pairs, n * sizeof(uint2), cudaMemcpyDeviceToHost);
                for (const uint2& p : chunk_pairs) bins_out.emplace_back(p.x, p.y < nvis ? prim_of[p.y] : 0xFFFFFFFEu);
            }
            renderer.Rasterizer(pCudaMesh, camFwd, cm);
            cudaDeviceSynchronize();
            renderer.m_BinQueues.ResetQueueSizes();
        }
    }
    renderer.PixelShader(ss, vs);
    const cudaError_t err = cudaDeviceSynchronize();
    if (err != cudaSuccess) {
        fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(err));
        return 4;
    }

    const size_t npx = (size_t)W * H;
    std::vector<uint32_t> colour(npx);
    std::vector<PixelShade> frags(npx);
    cudaMemcpy(colour.data(), renderer.m_CUDAWindowHelper.GetDev_FrameBuffer(), npx * 4u, cudaMemcpyDeviceToHost);
    cudaMemcpy(frags.data(), renderer.m_CUDAWindowHelper.GetDev_FragmentBuffer(), npx * sizeof(PixelShade),
               cudaMemcpyDeviceToHost);
    std::vector<float> z(npx);
    for (size_t i = 0; i < npx; ++i) z[i] = frags[i].zInterpolated;

    FILE* fo = fopen(argv[2], "wb");
    if (!fo) { perror("out"); return 2; }
    const uint32_t hdr[4] = {0x4F524247u, W, H, (uint32_t)total_visible};
    fwrite(hdr, 4, 4, fo);
    fwrite(colour.data(), 4, npx, fo);
    fwrite(z.data(), 4, npx, fo);
    const uint64_t np = bins_out.size();
    fwrite(&np, 8, 1, fo);
    for (const auto& p : bins_out) {
        const uint32_t v[2] = {p.first, p.second};
        fwrite(v, 4, 2, fo);
    }
    fclose(fo);
    cudaFree(d_pairs);
    cudaFree(d_count);
    printf("reference frame: %llu triangles, %llu visible, %llu bin pairs\n", (unsigned long long)total_tris,
           (unsigned long long)total_visible, (unsigned long long)np);
    return 0;
}
