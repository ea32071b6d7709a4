// gbr_draw.cu -- DrawTexture / DrawTextureGlobal (CUDARenderer.cu:1968-2012):
// a texture drawn straight into the colour buffer.
//
// gbr_draw_texture follows TextureTestKernel (CUDARenderer.cu:1565-1588): the
// window pixel's normalised position is looked up with the texture hardware
// -- a pitch-2D texture object with normalised coordinates, point filtering
// and the default (wrap) addressing, as CUDATexture::Create makes it
// (CUDATexture.cpp:24-64) -- and the texel's red and blue bytes are swapped.
// gbr_draw_texture_global follows DrawTextureGlobalKernel
// (CUDARenderer.cu:1590-1615): uv = pixel / window size (stretched) or /
// texture size, the shader's software sampler (point or the reference's
// "linear"), and the sampler's colour to colour32.  The reference's grids
// truncate (width / 16 blocks); every pixel is drawn here.  Depth and ids
// keep the last frame's values.
#include "gbr_device.cuh"
#include "gbr_internal.h"
#include "gbr_kernels.h"
#include "gbr_shade.cuh"

namespace gbr {

namespace {

__global__ void draw_texture_kernel(uint32_t* colour, cudaTextureObject_t tex, uint32_t width, uint32_t height) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= width || y >= height) return;
    const float u = __fdiv_rn((float)x, (float)width);
    const float v = __fdiv_rn((float)y, (float)height);
    const uint32_t t = tex2D<uint32_t>(tex, u, v);
    // swap the red and blue bytes (the RGBA union's r8 <-> b8)
    colour[x + y * width] = (t & 0xFF00FF00u) | ((t & 0xFFu) << 16) | ((t >> 16) & 0xFFu);
}

__global__ void draw_texture_global_kernel(uint32_t* colour, TexDev tex, int stretch, uint32_t sample, uint32_t width,
                                           uint32_t height) {
    const uint32_t x = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t y = blockIdx.y * blockDim.y + threadIdx.y;
    if (x >= width || y >= height) return;
    const float u = __fdiv_rn((float)x, (float)(stretch ? width : tex.w));
    const float v = __fdiv_rn((float)y, (float)(stretch ? height : tex.h));
    const F3 c = sample == 1u ? sample_linear(tex, u, v) : sample == 2u ? sample_bilinear(tex, u, v) : sample_point(tex, u, v);
    colour[x + y * width] = rgba_from_colour(c);
}

gbr_status texture_of(gbr_renderer* r, int32_t id, TexHost*& t) {
    if (!r) return fail(GBR_ERR_INVALID_ARG, "renderer is null");
    if (id < 0 || (size_t)id >= r->textures.size() || !r->textures[id].d_px)
        return fail(GBR_ERR_NOT_FOUND, "texture %d does not exist", id);
    t = &r->textures[id];
    return GBR_OK;
}

}  // namespace

void free_texture(TexHost& t) {
    if (t.tex_obj) cudaDestroyTextureObject((cudaTextureObject_t)t.tex_obj);
    cudaFree(t.d_pitched);
    cudaFree(t.d_px);
    t = TexHost();
}

}  // namespace gbr

using namespace gbr;

extern "C" {

gbr_status gbr_draw_texture(gbr_renderer* r, int32_t tex_id, void* stream) {
    TexHost* t = nullptr;
    gbr_status st = texture_of(r, tex_id, t);
    if (st != GBR_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    if (!t->tex_obj) {
        int dev = 0, align = 0;
        GBR_CUDA(cudaGetDevice(&dev));
        GBR_CUDA(cudaDeviceGetAttribute(&align, cudaDevAttrTexturePitchAlignment, dev));
        const size_t row = (size_t)t->w * 4u;
        const uint32_t* base = t->d_px;
        size_t pitch = row;
        if (align > 0 && row % (size_t)align != 0) {   // rows re-laid at the texture pitch
            GBR_CUDA(cudaMallocPitch((void**)&t->d_pitched, &pitch, row, t->h));
            GBR_CUDA(cudaMemcpy2D(t->d_pitched, pitch, t->d_px, row, row, t->h, cudaMemcpyDeviceToDevice));
            base = t->d_pitched;
        }
        cudaResourceDesc res;
        memset(&res, 0, sizeof res);
        res.resType = cudaResourceTypePitch2D;
        res.res.pitch2D.devPtr = const_cast<uint32_t*>(base);
        res.res.pitch2D.desc = cudaCreateChannelDesc<uint32_t>();
        res.res.pitch2D.width = t->w;
        res.res.pitch2D.height = t->h;
        res.res.pitch2D.pitchInBytes = pitch;
        cudaTextureDesc td;
        memset(&td, 0, sizeof td);
        td.normalizedCoords = 1;
        td.filterMode = cudaFilterModePoint;
        td.readMode = cudaReadModeElementType;
        cudaTextureObject_t obj = 0;
        GBR_CUDA(cudaCreateTextureObject(&obj, &res, &td, nullptr));
        t->tex_obj = (unsigned long long)obj;
    }
    const dim3 block(16, 16), grid((r->W + 15u) / 16u, (r->H + 15u) / 16u);
    draw_texture_kernel<<<grid, block, 0, s>>>(r->d_colour, (cudaTextureObject_t)t->tex_obj, r->W, r->H);
    GBR_CUDA(cudaGetLastError());
    r->drawn = true;
    r->dirty_valid = false;
    return GBR_OK;
}

gbr_status gbr_draw_texture_global(gbr_renderer* r, int32_t tex_id, int stretch_to_window, uint32_t sample,
                                   void* stream) {
    TexHost* t = nullptr;
    gbr_status st = texture_of(r, tex_id, t);
    if (st != GBR_OK) return st;
    if (sample > GBR_SAMPLE_BILINEAR) return fail(GBR_ERR_INVALID_ARG, "unknown sample state %u", sample);
    TexDev td;
    td.px = t->d_px;
    td.w = t->w;
    td.h = t->h;
    const dim3 block(16, 16), grid((r->W + 15u) / 16u, (r->H + 15u) / 16u);
    draw_texture_global_kernel<<<grid, block, 0, (cudaStream_t)stream>>>(r->d_colour, td, stretch_to_window != 0, sample,
                                                                        r->W, r->H);
    GBR_CUDA(cudaGetLastError());
    r->drawn = true;
    r->dirty_valid = false;
    return GBR_OK;
}

}  // extern "C"
