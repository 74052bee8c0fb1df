"""The drop-in boundary at link level: a C++ translation unit that declares GPView's CUDA entry
points exactly as the reference's includes/CUDAUtilities.h does (C linkage for the classify and
THRUST functions, C++ linkage for InitializeCUDA / CUDACheckErrors, which the application defines
itself in src/CUDAUtilities.cpp) links against libgpview.so in place of the GPViewCUDA library,
with every symbol resolved at load time.  The program runs its GPU calls only when asked, so the
test needs no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# The caller side as GPView's sources have it: the declarations of includes/CUDAUtilities.h:63-64,
# :72-74, :87-89 (signatures as the reference writes them), the application's own definitions of
# InitializeCUDA / CUDACheckErrors and THRUSTFindMax (src/CUDAUtilities.cpp:33-55, :121-132, in
# outline), and calls shaped like Object::ClassifyTessellationCUDA and its Level2 siblings.
CALLER = r"""
#include <cstdio>
#include <cuda_runtime.h>

void InitializeCUDA();
void CUDACheckErrors(char const* label = NULL);
extern "C" float THRUSTDeviceFindMax(float* dataCUDAPointer, int w, int h);
extern "C" float THRUSTDeviceFindMaxFloat4(float4* dataCUDAPointer, int numValues, float4* maxVal, int* maxLoc);
extern "C" void THRUSTDeviceMinMaxSort(float* minDataCUDAPointer, float* maxDataCUDAPointer, int* rowDataCUDAPointer, int n, float* minData, float* maxData, int* rowNumbers);
extern "C" int CUDAClassifyTessellation(float* trianglesCUDAData, int numTriangles, float* inOutCUDAData, int* voxelTriCountCUDAData, int* voxelTriIndexCUDAData, float3 objBoxMin, float3 objBoxMax, float3 boxExtents, int3 numDiv, int triBufferLen);
extern "C" int CUDAClassifyTessellationLevel2(float* trianglesCUDAData, float* level2InOutCUDAData, float* level2NormalCUDAData, float* level1MidPointCUDAData, int* level2IndexCUDAData, int* voxelTriCountCUDAData, int* level1TriFlatIndexCUDAData, int* level1TriFlatCUDAData, int numBoundary, int3 numDiv2, float3 boxExtentsLevel1, float3 boxExtentsLevel2);
extern "C" int CUDAClassifyInOutLevel2(float* trianglesCUDAData, float* level2InOutCUDAData, float* level1MidPointCUDAData, int* level2IndexCUDAData, int* voxelTriCountCUDAData, int* level1TriFlatIndexCUDAData, int* level1TriFlatCUDAData, int numBoundary, int3 numDiv, int3 numDiv2, float3 boxExtentsLevel1, float3 boxExtentsLevel2);

// the application's own definitions (C++ linkage), as src/CUDAUtilities.cpp has them
void CUDACheckErrors(char const* label) {
  cudaError_t e = cudaDeviceSynchronize();
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e != cudaSuccess) std::printf("CUDA Error: %s %s\n", label ? label : "", cudaGetErrorString(e));
}
void InitializeCUDA() { cudaSetDevice(0); CUDACheckErrors(" Init "); }
float THRUSTFindMax4(float* k1, float* k2, float* k3, float* k4, int w, int h) {
  return THRUSTDeviceFindMax(k1, w, h) + THRUSTDeviceFindMax(k2, w, h) +
         THRUSTDeviceFindMax(k3, w, h) + THRUSTDeviceFindMax(k4, w, h);
}

int main(int argc, char** argv) {
  if (argc < 2) { std::printf("linked\n"); return 0; }  // the GPU calls run only on request
  InitializeCUDA();
  float* tris = nullptr; float* inOut = nullptr; int* cnt = nullptr; int* idx = nullptr;
  cudaMalloc(&tris, 9 * sizeof(float)); cudaMalloc(&inOut, 64 * sizeof(float));
  cudaMalloc(&cnt, 64 * sizeof(int)); cudaMalloc(&idx, 64 * sizeof(int));
  cudaMemset(tris, 0, 9 * sizeof(float)); cudaMemset(inOut, 0, 64 * sizeof(float));
  cudaMemset(cnt, 0, 64 * sizeof(int));
  float3 mn = make_float3(-1, -1, -1), mx = make_float3(1, 1, 1), ext = make_float3(0.25f, 0.25f, 0.25f);
  int rc = CUDAClassifyTessellation(tris, 1, inOut, cnt, idx, mn, mx, ext, make_int3(4, 4, 4), 1);
  CUDACheckErrors("classify");
  float m = THRUSTFindMax4(inOut, inOut, inOut, inOut, 8, 8);
  float4 mv; int loc = -1;
  THRUSTDeviceFindMaxFloat4(reinterpret_cast<float4*>(inOut), 16, &mv, &loc);
  int rows[4];
  THRUSTDeviceMinMaxSort(inOut, inOut, cnt, 4, nullptr, nullptr, rows);
  (void)CUDAClassifyTessellationLevel2; (void)CUDAClassifyInOutLevel2;
  std::printf("rc=%d max=%g loc=%d\n", rc, m, loc);
  return rc == 1 ? 0 : 1;
}
"""


def _cuda_dirs():
    """(include dir, library dir) of the CUDA toolkit nvcc belongs to."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    root = os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    inc = os.path.join(root, "include")
    lib = next((d for d in (os.path.join(root, "lib64"), os.path.join(root, "lib"))
                if os.path.exists(os.path.join(d, "libcudart.so"))), None)
    return (inc if os.path.exists(os.path.join(inc, "cuda_runtime.h")) else None), lib


def test_reference_caller_links_and_loads(built, tmp_path):
    inc, cudalib = _cuda_dirs()
    if not inc or not cudalib or not shutil.which("g++"):
        pytest.skip("no CUDA toolkit or g++")
    src = tmp_path / "caller.cpp"
    src.write_text(CALLER)
    exe = tmp_path / "caller"
    libdir = os.path.join(ROOT, "gpview_gb300")
    # the application links the CUDA runtime itself (its own cudaMalloc, cudaMemcpy, ...)
    cmd = ["g++", "-std=c++17", "-I", inc, str(src), "-L", libdir, "-lgpview", "-L", cudalib,
           "-lcudart", f"-Wl,-rpath,{libdir}:{cudalib}", "-Wl,-z,now", "-Wl,--no-undefined",
           "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    # every symbol the caller needs is resolved when the program loads (-z now)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and "linked" in r.stdout, r.stderr
