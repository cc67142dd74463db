// Stiffness apply without device allocation, for callers that cannot call
// cudaMalloc: applications whose device memory is owned by another
// allocator (a framework's caching pool, a fixed arena reserved at start-up)
// and real-time loops that must not hit cudaMalloc/cudaFree, which can block
// and, for cudaFree, synchronise the whole device.
//
// f = K u for the structured mesh of unit cubes split into six Kuhn
// tetrahedra (mu_r = 1), in FP32, on device arrays the caller owns.  The
// per-tetrahedron curl scratch lives in a file-scope __device__ array of
// fixed size, so this entry point allocates nothing; the mesh topology is
// derived arithmetically instead of being read from incidence lists.  The
// operations and their order match ems_tetfem_apply_stiffness in FP32.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "ems_internal.hpp"

namespace ems {
void record_error(const std::string &msg);
}

namespace {

// Maximum mesh size: 2^20 tetrahedra (174,762 cubes, e.g. 55^3); the scratch
// holds 3 floats per tetrahedron, 12 MiB, resident on every device that loads
// the library until the process exits.
constexpr size_t kStaticMaxTets = (size_t)1 << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) float g_tet_curl_scratch[3 * kStaticMaxTets];

__constant__ int s_perm[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
__constant__ int s_loc[6][2] = {{0, 1}, {0, 2}, {0, 3}, {1, 2}, {1, 3}, {2, 3}};
__constant__ int s_dir[7][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {1, 1, 1}};

std::mutex g_mu;
float *g_scratch[kMaxDevices] = {};

// vertex offset of vertex `v` of Kuhn tetrahedron type p
__device__ __forceinline__ void kuhn_vert(int p, int v, int o[3])
{
    o[0] = o[1] = o[2] = 0;
    if (v >= 1) o[s_perm[p][0]] = 1;
    if (v >= 2) o[s_perm[p][1]] = 1;
    if (v >= 3) o[s_perm[p][2]] = 1;
}

// gradient of barycentric coordinate `v` (unit cube)
__device__ __forceinline__ void kuhn_grad(int p, int v, float g[3])
{
    g[0] = g[1] = g[2] = 0.f;
    if (v == 0) g[s_perm[p][0]] = -1.f;
    else if (v == 3) g[s_perm[p][2]] = 1.f;
    else { g[s_perm[p][v - 1]] = 1.f; g[s_perm[p][v]] = -1.f; }
}

__device__ __forceinline__ void kuhn_curl(int p, int l, float c[3])
{
    float gm[3], gn[3];
    kuhn_grad(p, s_loc[l][0], gm);
    kuhn_grad(p, s_loc[l][1], gn);
    c[0] = 2.f * (gm[1] * gn[2] - gm[2] * gn[1]);
    c[1] = 2.f * (gm[2] * gn[0] - gm[0] * gn[2]);
    c[2] = 2.f * (gm[0] * gn[1] - gm[1] * gn[0]);
}

__device__ __forceinline__ int dir_of(const int a[3], const int b[3])
{
    for (int d = 0; d < 7; ++d)
        if (b[0] - a[0] == s_dir[d][0] && b[1] - a[1] == s_dir[d][1] && b[2] - a[2] == s_dir[d][2]) return d;
    return -1;
}

// B_t = 1/6 * sum_l u[slot(t,l)] curl(w_l), into the static scratch
__global__ void static_curl_kernel(int nx, int ny, int nz, const float *__restrict__ u, float *__restrict__ B)
{
    size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t ntet = 6 * (size_t)nx * ny * nz;
    if (t >= ntet) return;
    int p = (int)(t % 6);
    size_t cell = t / 6;
    int ci = (int)(cell % nx), cj = (int)((cell / nx) % ny), ck = (int)(cell / ((size_t)nx * ny));
    float c0 = 0.f, c1 = 0.f, c2 = 0.f;
    for (int l = 0; l < 6; ++l) {
        int vm[3], vn[3];
        kuhn_vert(p, s_loc[l][0], vm);
        kuhn_vert(p, s_loc[l][1], vn);
        int d = dir_of(vm, vn);
        size_t node = (size_t)(ci + vm[0]) + (size_t)(nx + 1) * ((size_t)(cj + vm[1]) + (size_t)(ny + 1) * (ck + vm[2]));
        float uv = u[7 * node + d], cr[3];
        kuhn_curl(p, l, cr);
        c0 = fmaf(uv, cr[0], c0);
        c1 = fmaf(uv, cr[1], c1);
        c2 = fmaf(uv, cr[2], c2);
    }
    const float s = (float)(1.0 / 6.0);
    B[3 * t] = s * c0;
    B[3 * t + 1] = s * c1;
    B[3 * t + 2] = s * c2;
}

// f_e = sum over the tetrahedra containing edge slot e of B_t . curl(w_l),
// visited in increasing tetrahedron index (the incidence-list order of the
// allocating path); zero on unused and PEC slots.
__global__ void static_gather_kernel(int nx, int ny, int nz, const float *__restrict__ B, float *__restrict__ f)
{
    size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    size_t nslot = 7 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    if (e >= nslot) return;
    int d = (int)(e % 7);
    size_t v = e / 7;
    int a[3] = {(int)(v % (nx + 1)), (int)((v / (nx + 1)) % (ny + 1)), (int)(v / ((size_t)(nx + 1) * (ny + 1)))};
    const int lim[3] = {nx, ny, nz};
    int b[3] = {a[0] + s_dir[d][0], a[1] + s_dir[d][1], a[2] + s_dir[d][2]};
    bool pec = b[0] > nx || b[1] > ny || b[2] > nz;
    for (int q = 0; q < 3 && !pec; ++q)
        if (a[q] == b[q] && (a[q] == 0 || a[q] == lim[q])) pec = true;
    float acc = 0.f;
    if (!pec)
        for (int dz = 1; dz >= 0; --dz)
            for (int dy = 1; dy >= 0; --dy)
                for (int dx = 1; dx >= 0; --dx) {
                    int c[3] = {a[0] - dx, a[1] - dy, a[2] - dz};
                    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= nx || c[1] >= ny || c[2] >= nz) continue;
                    size_t cell = (size_t)c[0] + (size_t)nx * ((size_t)c[1] + (size_t)ny * c[2]);
                    for (int p = 0; p < 6; ++p)
                        for (int l = 0; l < 6; ++l) {
                            int vm[3], vn[3];
                            kuhn_vert(p, s_loc[l][0], vm);
                            if (vm[0] != dx || vm[1] != dy || vm[2] != dz) continue;
                            kuhn_vert(p, s_loc[l][1], vn);
                            if (dir_of(vm, vn) != d) continue;
                            size_t t = 6 * cell + p;
                            float cr[3];
                            kuhn_curl(p, l, cr);
                            acc = fmaf(B[3 * t], cr[0], acc);
                            acc = fmaf(B[3 * t + 1], cr[1], acc);
                            acc = fmaf(B[3 * t + 2], cr[2], acc);
                        }
                }
    f[e] = acc;
}

}  // namespace

extern "C" int ems_tet_stiffness_apply_static(const int cells[3], const float *u, float *f, void *stream)
{
    if (!cells || !u || !f) {
        ems::record_error("cells, u and f are required");
        return EMS_ERR_INVALID_ARGUMENT;
    }
    const int nx = cells[0], ny = cells[1], nz = cells[2];
    if (nx < 1 || ny < 1 || nz < 1) {
        ems::record_error("cell counts must be positive");
        return EMS_ERR_INVALID_ARGUMENT;
    }
    const size_t ntet = 6 * (size_t)nx * ny * nz;
    if (ntet > kStaticMaxTets) {
        ems::record_error("mesh of " + std::to_string(ntet) + " tetrahedra exceeds the fixed scratch of " +
                          std::to_string(kStaticMaxTets) + " tetrahedra of ems_tet_stiffness_apply_static");
        return EMS_ERR_INVALID_ARGUMENT;
    }
    int dev = 0;
    cudaError_t rc = cudaGetDevice(&dev);
    if (rc != cudaSuccess) {
        ems::record_error(std::string("cudaGetDevice: ") + cudaGetErrorString(rc));
        return EMS_ERR_CUDA;
    }
    if (dev < 0 || dev >= kMaxDevices) {
        ems::record_error("device index " + std::to_string(dev) + " beyond the " + std::to_string(kMaxDevices) +
                          " devices ems_tet_stiffness_apply_static keeps scratch addresses for");
        return EMS_ERR_INVALID_ARGUMENT;
    }
    float *scratch = nullptr;
    {
        // once per device, with that device current: the host-side name of the
        // array is not a device address, so look the address up.  The address
        // is kept for the life of the process; a cudaDeviceReset of the device
        // unloads the module that holds the array, so the library must not be
        // used on a device after the process reset it.
        std::lock_guard<std::mutex> lock(g_mu);
        if (!g_scratch[dev]) {
            rc = cudaGetSymbolAddress((void **)&scratch, g_tet_curl_scratch);
            if (rc != cudaSuccess) {
                ems::record_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(rc));
                return EMS_ERR_CUDA;
            }
            g_scratch[dev] = scratch;
        }
        scratch = g_scratch[dev];
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const size_t nslot = 7 * (size_t)(nx + 1) * (ny + 1) * (nz + 1);
    static_curl_kernel<<<(unsigned)((ntet + 255) / 256), 256, 0, s>>>(nx, ny, nz, u, scratch);
    static_gather_kernel<<<(unsigned)((nslot + 255) / 256), 256, 0, s>>>(nx, ny, nz, scratch, f);
    rc = cudaGetLastError();
    if (rc != cudaSuccess) {
        ems::record_error(std::string("kernel launch: ") + cudaGetErrorString(rc));
        return EMS_ERR_CUDA;
    }
    return EMS_OK;
}
