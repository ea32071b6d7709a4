// sdl_stubs.cpp -- headless stand-ins for the SDL2 / SDL2_image entry points
// the reference's renderer sources link against (TEST INFRASTRUCTURE ONLY).
// No window, surface or event exists: texture loading is done by the
// harness from memory, so IMG_Load is never reached.
#include <SDL.h>
#include <SDL_image.h>

extern "C" {
SDL_Surface* IMG_Load(const char*) { return nullptr; }
void SDL_FreeSurface(SDL_Surface*) {}
int SDL_LockSurface(SDL_Surface*) { return 0; }
void SDL_UnlockSurface(SDL_Surface*) {}
int SDL_UpperBlit(SDL_Surface*, const SDL_Rect*, SDL_Surface*, SDL_Rect*) { return 0; }
int SDL_UpdateWindowSurface(SDL_Window*) { return 0; }
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
