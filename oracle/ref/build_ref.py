"""Recipe that builds the reference's own CUDARenderer as a GPU oracle.

TEST INFRASTRUCTURE ONLY.  stage() copies the reference sources
(CustomCUDARasterizer/*.h/.cpp/.cu/.cuh and the SDL2 headers of 3rdParty/)
from the read-only reference checkout into oracle/_ref/src/ (git-ignored, so
the copy never enters history but travels to the GPU machine) and applies the
patches listed in PATCHES, each of which must match exactly once:

  P1-P5  compatibility with nvcc 13 / g++ 13 (std::powf, flexible array
         members in unions, a member-name typo, cudaDeviceProp fields removed
         in CUDA 13, reinterpret_cast of a temporary);
  P6     Clear/PixelShader grids rounded up instead of truncated, so rows
         past the last full 32- or 16-pixel block are cleared and shaded;
  P7     RA_PerTileKernel clamps its pixel range to the screen (the unpatched
         kernel writes past the buffers when the last bin row or column
         extends beyond the screen);
  P8     the two spin locks (bin-queue insert, per-pixel depth lock) give up
         after 2^26 attempts instead of spinning forever;
  P9     CUDARenderer's private members are made public for the harness.

build() compiles oracle/ref/ref_harness.cu (which includes the staged
CUDARenderer.cu) with the staged host sources and the SDL stubs into
oracle/_ref/ref_harness with nvcc for sm_103a, using nvcc's default
floating-point contraction for device code (as the reference build) and
-ffp-contract=off for host code (as MSVC, which does not fuse).
No source of the reference checkout is modified.
"""
import os
import re
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
OUT = os.path.join(ORACLE, "_ref")
SRC = os.path.join(OUT, "src")
# The reference checkout: GBR_REFERENCE_ROOT, else a "reference" directory
# beside this repository's checkout (where the build machine keeps it).
REPO = os.path.dirname(ORACLE)
REF = os.environ.get("GBR_REFERENCE_ROOT") or os.path.join(os.path.dirname(REPO), "reference")
CCR = os.path.join(REF, "CustomCUDARasterizer")


def reference_present() -> bool:
    """Whether the reference's sources are on this machine (the recipe
    builds nothing otherwise)."""
    return os.path.isdir(CCR)
BIN = os.path.join(OUT, "ref_harness")

HOST_SOURCES = ["CUDAMesh.cpp", "CUDATexture.cpp", "CUDATextureManager.cpp", "Mesh.cpp", "SceneGraph.cpp",
                "SceneManager.cpp", "Camera.cpp", "Resolution.cpp", "CUDABenchMarker.cpp", "Light.cpp",
                "DirectionalLight.cpp", "PointLight.cpp", "EventManager.cpp"]

# (file, pattern, replacement, is_regex)
PATCHES = [
    ("RGBColor.h", "std::powf", "powf", "all"),                                                      # P1
    ("Structs.h", r"struct RenderData // size == 35\n\{.*?\n\};\n", "", True),                       # P2
    ("Structs.h", "struct TriangleIdxBb // size == 5\n{\n\tunion\n\t{\n\t\tunsigned int idx[];",
     "struct TriangleIdxBb // size == 5\n{\n\tunion\n\t{\n\t\tunsigned int idx[3];", False),         # P2
    ("CUDAAtomicQueue.cuh", "(void**)&m_Dev_QueueSizeMutex, 4)", "(void**)&m_Dev_QueueSizeMutexBuffer, 4)", False),  # P3
    ("CUDAAtomicQueue.cuh", "cudaFree(m_Dev_QueueSizeMutex));\n\t\tCheckErrorCuda(cudaFree(m_Dev_QueueSize));",
     "cudaFree(m_Dev_QueueSizeMutexBuffer));\n\t\tCheckErrorCuda(cudaFree(m_Dev_QueueSize));", False),   # P3
    ("CUDARenderer.cu", r"CPU_CALLABLE\nvoid CUDARenderer::DisplayGPUSpecs\(int deviceId\)\n\{.*?\n\}\n\nCPU_CALLABLE\nvoid CUDARenderer::LoadScene",
     "CPU_CALLABLE\nvoid CUDARenderer::DisplayGPUSpecs(int deviceId)\n{\n\t(void)deviceId;\n}\n\nCPU_CALLABLE\nvoid CUDARenderer::LoadScene", True),  # P4
    ("CUDAROPs.cu", "\treturn reinterpret_cast<RGBColor&>(InterpolateVector(",
     "\tconst FVector3 v = InterpolateVector(", False),                                              # P5
    ("CUDAROPs.cu", "\t\tweights, invDepths));\n}", "\t\tweights, invDepths);\n\treturn RGBColor{ v.x, v.y, v.z };\n}", False),  # P5
    # P6: round the Clear/PixelShader grids up
    ("CUDARenderer.cu", "const dim3 numBlocks{ width / numThreadsPerBlock.x, height / numThreadsPerBlock.y };",
     "const dim3 numBlocks{ (width + numThreadsPerBlock.x - 1) / numThreadsPerBlock.x, (height + numThreadsPerBlock.y - 1) / numThreadsPerBlock.y };",
     "all"),
    # P7: clamp the per-thread pixel range of RA_PerTileKernel to the screen
    ("CUDARenderer.cu", "\tbb.yMax = ClampFast(bb.yMax, (short)minY, (short)maxY);\n\n#ifdef FINERASTER_SHAREDMEM",
     "\tbb.yMax = ClampFast(bb.yMax, (short)minY, (short)maxY);\n"
     "\tbb.xMax = ClampFast(bb.xMax, (short)0, (short)width);\n"
     "\tbb.yMax = ClampFast(bb.yMax, (short)0, (short)height);\n\n#ifdef FINERASTER_SHAREDMEM", False),
    # P8: bounded spin locks
    ("CUDAAtomicQueue.cuh", "\tvoid Insert(T* dev_Queue, unsigned int& dev_QueueSize, int& dev_QueueSizeMutex, unsigned int queueMaxSize, T data)\n\t{\n\t\tbool isDone = false;\n\t\tdo",
     "\tvoid Insert(T* dev_Queue, unsigned int& dev_QueueSize, int& dev_QueueSizeMutex, unsigned int queueMaxSize, T data)\n\t{\n\t\tbool isDone = false;\n\t\tunsigned int spinGuard = 0;\n\t\tdo", False),
    ("CUDAAtomicQueue.cuh", "\t\t\t\tdev_QueueSizeMutex = 0;\n\t\t\t\t//end of critical section\n\t\t\t}\n\t\t} while (!isDone);\n\t}\n\n\ttemplate <typename T>\n\tGPU_CALLABLE GPU_INLINE static\n\t//Only valid",
     "\t\t\t\tdev_QueueSizeMutex = 0;\n\t\t\t\t//end of critical section\n\t\t\t}\n\t\t} while (!isDone && ++spinGuard < (1u << 26));\n\t}\n\n\ttemplate <typename T>\n\tGPU_CALLABLE GPU_INLINE static\n\t//Only valid", False),
    ("CUDAROPs.cu", "\t//Update depthbuffer atomically\n\tbool isDone = false;\n\tdo",
     "\t//Update depthbuffer atomically\n\tbool isDone = false;\n\tunsigned int spinGuard = 0;\n\tdo", False),
    ("CUDAROPs.cu", "\t\t\tdev_DepthMutexBuffer[pixelIdx] = 0;\n\t\t\t//end of critical section\n\t\t}\n\t} while (!isDone);",
     "\t\t\tdev_DepthMutexBuffer[pixelIdx] = 0;\n\t\t\t//end of critical section\n\t\t}\n\t} while (!isDone && ++spinGuard < (1u << 26));", False),
    # P9
    ("CUDARenderer.h", "private:", "public:", "all"),
    # E1-E4: the CPU renderer (ERenderer.cpp, absent from the reference's
    # project) against the current Mesh / SceneManager API: raw vertex and
    # index buffers, GetNum* counts, GetWorldConst, the visualisation state
    # instead of IsDepthColour, textures looked up by the harness
    ("ERenderer.cpp", "\t\tconst std::vector<IVertex>& vertexBuffer = pMesh->GetVertexBuffer();\n"
                      "\t\tconst unsigned int numVertices = pMesh->GetVertexAmount();\n"
                      "\t\tconst std::vector<unsigned int>& indexBuffer = pMesh->GetIndexBuffer();\n"
                      "\t\tconst unsigned int numIndices = pMesh->GetIndexAmount();\n"
                      "\t\tm_pTextures = &pMesh->GetTextures();",
     "\t\tconst IVertex* vertexBuffer = pMesh->GetVertexBuffer();\n"
     "\t\tconst unsigned int numVertices = pMesh->GetNumVertices();\n"
     "\t\tconst unsigned int* indexBuffer = pMesh->GetIndexBuffer();\n"
     "\t\tconst unsigned int numIndices = pMesh->GetNumIndices();\n"
     "\t\tm_pTextures = &ErefTexturesOf(pMesh);", False),                                           # E1
    ("ERenderer.cpp", "GetNDCMeshVertices(vertexBuffer, viewProjectionMatrix, pMesh->GetWorldMatrix())",
     "GetNDCMeshVertices(reinterpret_cast<const float*>(vertexBuffer), numVertices, viewProjectionMatrix, "
     "pMesh->GetWorldConst())", False),                                                               # E2
    ("ERenderer.cpp", "!sm.IsDepthColour()", "!(sm.GetVisualisationState() == VisualisationState::Depth)", "all"),  # E3
    ("ERenderer.cpp", '#include "CullingMode.h"\n',
     '#include "CullingMode.h"\n#include "VisualisationState.h"\n#include "SampleState.h"\n'
     "const Textures& ErefTexturesOf(const Mesh* pMesh);\n", False),                                # E4
    ("SceneManager.h", "private:", "public:", "all"),                                                  # E5
    ("ERenderer.h", "\tprivate:", "\tpublic:", "all"),                                                 # E6
]

ERENDERER_SOURCES = ["ERenderer.cpp", "Mesh.cpp", "SceneGraph.cpp", "SceneManager.cpp", "Camera.cpp", "Texture.cpp",
                     "Light.cpp", "DirectionalLight.cpp", "PointLight.cpp", "EventManager.cpp"]
EREF_BIN = os.path.join(OUT, "eref_harness")


def _apply(text, pat, rep, mode, name):
    if mode is True:
        new, n = re.subn(pat, lambda m: rep, text, count=1, flags=re.S)
    elif mode == "all":
        n = text.count(pat)
        new = text.replace(pat, rep)
    else:
        n = text.count(pat)
        new = text.replace(pat, rep, 1)
    if n < 1 or (mode is False and n != 1):
        raise RuntimeError(f"patch for {name} matched {n} times: {pat[:60]!r}")
    return new


def stage(force: bool = False) -> str:
    """Copy and patch the reference sources into oracle/_ref/src."""
    if not os.path.isdir(CCR):
        raise FileNotFoundError(f"reference sources not found at {CCR}")
    stamp = os.path.join(SRC, ".staged")
    if os.path.exists(stamp) and not force and os.path.getmtime(stamp) >= os.path.getmtime(__file__):
        return SRC
    if os.path.isdir(SRC):
        shutil.rmtree(SRC)
    os.makedirs(SRC)
    for f in os.listdir(CCR):
        if f.endswith((".h", ".cpp", ".cu", ".cuh")):
            shutil.copy2(os.path.join(CCR, f), os.path.join(SRC, f))
    for d in ("sdl2-2.0.9", "sdl2_image-2.0.5"):
        shutil.copytree(os.path.join(REF, "3rdParty", "include", d), os.path.join(SRC, "sdl", d))
    by_file = {}
    for f, pat, rep, mode in PATCHES:
        by_file.setdefault(f, []).append((pat, rep, mode))
    for f, plist in by_file.items():
        p = os.path.join(SRC, f)
        text = open(p, encoding="latin-1").read()
        for pat, rep, mode in plist:
            text = _apply(text, pat, rep, mode, f)
        open(p, "w", encoding="latin-1").write(text)
    open(stamp, "w").write("staged\n")
    return SRC


def nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def build(force: bool = False) -> str:
    """Compile the harness against the staged sources (stage() must have run,
    here or on the machine the staged copy came from)."""
    if not os.path.isdir(SRC):
        stage()
    inputs = [os.path.join(HERE, "ref_harness.cu"), os.path.join(HERE, "sdl_stubs.cpp"), os.path.join(SRC, ".staged")]
    if not force and os.path.exists(BIN) and all(os.path.getmtime(BIN) >= os.path.getmtime(i) for i in inputs):
        return BIN
    inc = ["-I", SRC, "-I", os.path.join(SRC, "sdl", "sdl2-2.0.9"), "-I", os.path.join(SRC, "sdl", "sdl2_image-2.0.5")]
    cmd = [nvcc(), "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-w",
           "-Xcompiler", "-ffp-contract=off", "--expt-relaxed-constexpr", "-include", "cstring", *inc,
           os.path.join(HERE, "ref_harness.cu"), os.path.join(HERE, "sdl_stubs.cpp"),
           *[os.path.join(SRC, f) for f in HOST_SOURCES], "-o", BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(BIN + ".tmp", BIN)
    return BIN


def build_erenderer(force: bool = False) -> str:
    """Compile oracle/ref/eref_harness.cpp with the reference's CPU renderer
    (ERenderer.cpp and the scene classes it uses, staged and patched E1-E5)
    and headless SDL stand-ins into oracle/_ref/eref_harness, with g++ at
    -O2 and no floating-point contraction (the reference's MSVC build does
    not fuse)."""
    if not os.path.isdir(SRC):
        stage()
    inputs = [os.path.join(HERE, "eref_harness.cpp"), os.path.join(HERE, "eref_stubs.cpp"), os.path.join(SRC, ".staged")]
    if not force and os.path.exists(EREF_BIN) and all(os.path.getmtime(EREF_BIN) >= os.path.getmtime(i) for i in inputs):
        return EREF_BIN
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    inc = ["-I", SRC, "-I", os.path.join(SRC, "sdl", "sdl2-2.0.9"), "-I", os.path.join(SRC, "sdl", "sdl2_image-2.0.5"),
           "-I", cuda_inc]
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-w", "-ffp-contract=off", "-include", "cstring", *inc,
           os.path.join(HERE, "eref_harness.cpp"), os.path.join(HERE, "eref_stubs.cpp"),
           *[os.path.join(SRC, f) for f in ERENDERER_SOURCES], "-lpthread", "-o", EREF_BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(EREF_BIN + ".tmp", EREF_BIN)
    return EREF_BIN


OBJ_BIN = os.path.join(OUT, "obj_harness")


def build_objparser(force: bool = False) -> str:
    """Compile oracle/ref/obj_harness.cpp with the reference's ObjParser.cpp
    (staged, unpatched) into oracle/_ref/obj_harness, with g++ at -O2 and no
    floating-point contraction."""
    if not os.path.isdir(SRC):
        stage()
    inputs = [os.path.join(HERE, "obj_harness.cpp"), os.path.join(SRC, ".staged")]
    if not force and os.path.exists(OBJ_BIN) and all(os.path.getmtime(OBJ_BIN) >= os.path.getmtime(i) for i in inputs):
        return OBJ_BIN
    cuda_inc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")
    inc = ["-I", SRC, "-I", os.path.join(SRC, "sdl", "sdl2-2.0.9"), "-I", os.path.join(SRC, "sdl", "sdl2_image-2.0.5"),
           "-I", cuda_inc]
    cmd = [os.environ.get("CXX", "g++"), "-O2", "-std=c++17", "-w", "-ffp-contract=off", "-include", "cstring", *inc,
           os.path.join(HERE, "obj_harness.cpp"), os.path.join(SRC, "ObjParser.cpp"), "-o", OBJ_BIN + ".tmp"]
    subprocess.run(cmd, check=True)
    os.replace(OBJ_BIN + ".tmp", OBJ_BIN)
    return OBJ_BIN


if __name__ == "__main__":
    if "--stage" in sys.argv or os.path.isdir(CCR):
        stage(force="--force" in sys.argv)
    print(build(force="--force" in sys.argv))
    print(build_erenderer(force="--force" in sys.argv))
