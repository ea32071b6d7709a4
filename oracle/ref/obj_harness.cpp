// obj_harness.cpp -- runs the reference's ObjParser on a file (TEST
// INFRASTRUCTURE ONLY: it produces the golden OBJ fixtures the parser
// restatements are pinned to).
//
//   obj_harness FILE INVERT_Y OUT
//
// OpenFile + SetInvertYAxis + ReadFromObjFile (the pointer form main.cpp
// uses, ObjParser.cpp:100-108, 216-355) and writes OUT: uint32 vertex
// count (the largest index + 1: the reference reports the face count in
// some branches), uint32 index count, int32 vertex type, the vertices
// (56-byte IVertex) and the indices.  The global array new is replaced by
// a zero-filling one, so the fields the reference leaves unset (IVertex()
// is "purposely uninitialized") read as 0 instead of heap garbage.
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <new>

#include "ObjParser.h"

void* operator new[](std::size_t n) {
    void* p = std::calloc(n ? n : 1, 1);
    if (!p) throw std::bad_alloc();
    return p;
}
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete[](void* p, std::size_t) noexcept { std::free(p); }

int main(int argc, char** argv) {
    if (argc != 4) {
        std::fprintf(stderr, "usage: obj_harness FILE INVERT_Y OUT\n");
        return 2;
    }
    ObjParser parser{};
    if (!parser.OpenFile(argv[1])) {
        std::fprintf(stderr, "cannot open %s\n", argv[1]);
        return 1;
    }
    parser.SetInvertYAxis(std::atoi(argv[2]) != 0);
    IVertex* vertices = nullptr;
    unsigned int* indices = nullptr;
    unsigned int num_vertices = 0, num_indices = 0;
    short type = 0;
    parser.ReadFromObjFile(vertices, num_vertices, indices, num_indices, type);
    uint32_t used = 0;
    for (unsigned int i = 0; i < num_indices; ++i)
        if (indices[i] + 1u > used) used = indices[i] + 1u;
    FILE* f = std::fopen(argv[3], "wb");
    if (!f) return 1;
    const uint32_t ni = num_indices;
    const int32_t vt = type;
    std::fwrite(&used, 4, 1, f);
    std::fwrite(&ni, 4, 1, f);
    std::fwrite(&vt, 4, 1, f);
    static_assert(sizeof(IVertex) == 56, "IVertex is 56 bytes");
    std::fwrite(vertices, sizeof(IVertex), used, f);
    std::fwrite(indices, 4, ni, f);
    std::fclose(f);
    delete[] vertices;
    delete[] indices;
    return 0;
}
