// eref_stubs.cpp -- headless stand-ins for the SDL2 / SDL2_image entry
// points the reference's CPU renderer (ERenderer.cpp, Texture.cpp) links
// against (TEST INFRASTRUCTURE ONLY: the timed CPU baseline).
//
// There is no window: the "window" is a size, its surface a plain buffer.
// Back-buffer pixels are packed 0x00RRGGBB (SDL_MapRGB); textures are RGBA8
// words with byte 0 = red (SDL_GetRGB), registered by name from memory so
// that Texture's IMG_Load(path) finds them.
#include <SDL.h>
#include <SDL_image.h>

#include <cstdlib>
#include <cstring>
#include <map>
#include <string>

namespace {
int g_win_w = 0, g_win_h = 0;
SDL_PixelFormat g_format = {};
SDL_Surface g_front = {};
std::map<std::string, SDL_Surface*> g_images;

SDL_Surface* make_surface(int w, int h, const void* pixels) {
    SDL_Surface* s = static_cast<SDL_Surface*>(std::calloc(1, sizeof(SDL_Surface)));
    g_format.BitsPerPixel = 32;
    g_format.BytesPerPixel = 4;
    s->format = &g_format;
    s->w = w;
    s->h = h;
    s->pitch = 4 * w;
    s->pixels = std::calloc((size_t)w * h, 4);
    if (pixels) std::memcpy(s->pixels, pixels, (size_t)w * h * 4);
    s->refcount = 1;
    return s;
}
}  // namespace

// Harness side.
void eref_set_window_size(int w, int h) {
    g_win_w = w;
    g_win_h = h;
}
void eref_register_image(const char* name, const void* rgba8, int w, int h) {
    g_images[name] = make_surface(w, h, rgba8);
}
const uint32_t* eref_surface_pixels(SDL_Surface* s) { return static_cast<const uint32_t*>(s->pixels); }

extern "C" {
SDL_Surface* IMG_Load(const char* file) {
    auto it = g_images.find(file ? file : "");
    return it == g_images.end() ? nullptr : it->second;
}
void SDL_FreeSurface(SDL_Surface*) {}   // registered images and the back buffer live until exit
int SDL_LockSurface(SDL_Surface*) { return 0; }
void SDL_UnlockSurface(SDL_Surface*) {}
int SDL_UpperBlit(SDL_Surface*, const SDL_Rect*, SDL_Surface*, SDL_Rect*) { return 0; }
int SDL_UpdateWindowSurface(SDL_Window*) { return 0; }
SDL_Surface* SDL_GetWindowSurface(SDL_Window*) { return &g_front; }
void SDL_GetWindowSize(SDL_Window*, int* w, int* h) {
    if (w) *w = g_win_w;
    if (h) *h = g_win_h;
}
SDL_Surface* SDL_CreateRGBSurface(Uint32, int width, int height, int, Uint32, Uint32, Uint32, Uint32) {
    return make_surface(width, height, nullptr);
}
Uint32 SDL_MapRGB(const SDL_PixelFormat*, Uint8 r, Uint8 g, Uint8 b) {
    return ((Uint32)r << 16) | ((Uint32)g << 8) | (Uint32)b;
}
void SDL_GetRGB(Uint32 pixel, const SDL_PixelFormat*, Uint8* r, Uint8* g, Uint8* b) {
    *r = (Uint8)(pixel & 0xFFu);
    *g = (Uint8)((pixel >> 8) & 0xFFu);
    *b = (Uint8)((pixel >> 16) & 0xFFu);
}
SDL_RWops* SDL_RWFromFile(const char*, const char*) { return nullptr; }
int SDL_SaveBMP_RW(SDL_Surface*, SDL_RWops*, int) { return -1; }
// input (EventManager.cpp, linked through SceneManager's key toggles)
int SDL_PollEvent(SDL_Event*) { return 0; }
const Uint8* SDL_GetKeyboardState(int* numkeys) {
    static Uint8 keys[512] = {0};
    if (numkeys) *numkeys = 512;
    return keys;
}
SDL_bool SDL_GetRelativeMouseMode(void) { return SDL_FALSE; }
int SDL_SetRelativeMouseMode(SDL_bool) { return 0; }
Uint32 SDL_GetRelativeMouseState(int* x, int* y) {
    if (x) *x = 0;
    if (y) *y = 0;
    return 0;
}
}
