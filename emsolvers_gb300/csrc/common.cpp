// Shared plumbing: device buffers, handle base, element-matrix CSV reading
// and the reference's file-name number format.
#include <cuda_runtime.h>

#include <cmath>
#include <fstream>
#include <iomanip>
#include <sstream>

#include "ems_internal.hpp"

namespace ems {

void DevBuf::alloc(size_t b)
{
    release();
    if (b == 0) b = 16;
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, b);
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw Error{e == cudaErrorMemoryAllocation ? EMS_ERR_OUT_OF_MEMORY : EMS_ERR_CUDA,
                    std::string("cudaMalloc(") + std::to_string(b) + "): " + cudaGetErrorString(e)};
    }
    p = q;
    bytes = b;
}

void DevBuf::ensure(size_t b)
{
    if (p && bytes == (b == 0 ? 16 : b)) return;
    alloc(b);
}

void DevBuf::zero(cudaStream_t s) { EMS_CUDA(cudaMemsetAsync(p, 0, bytes, s)); }

void DevBuf::release()
{
    if (p) cudaFree(p);
    p = nullptr;
    bytes = 0;
}

Sim::~Sim()
{
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (stream) cudaStreamDestroy(stream);
}

void Sim::init_stream()
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        throw Error{EMS_ERR_CUDA, "no CUDA device available"};
    }
    EMS_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
    EMS_CUDA(cudaEventCreate(&ev0));
    EMS_CUDA(cudaEventCreate(&ev1));
}

// fem_v2/fem_simulation.cpp:1477-1493: trim spaces and quotes, "a/b" -> a/b.
double parse_value(const std::string &str)
{
    size_t start = str.find_first_not_of(" \t\r\n\"");
    size_t end = str.find_last_not_of(" \t\r\n\"");
    if (start == std::string::npos) return 0.0;
    std::string t = str.substr(start, end - start + 1);
    size_t slash = t.find('/');
    try {
        if (slash != std::string::npos) return std::stod(t.substr(0, slash)) / std::stod(t.substr(slash + 1));
        return std::stod(t);
    } catch (const std::exception &) {
        throw Error{EMS_ERR_IO, "malformed matrix entry '" + t + "'"};
    }
}

// fem_v2/fem_simulation.cpp:1495-1524: one row per line, comma separated.
std::vector<std::vector<double>> load_matrix_csv(const std::string &path)
{
    std::ifstream f(path);
    if (!f.is_open()) throw Error{EMS_ERR_IO, "cannot open file: " + path};
    std::vector<std::vector<double>> m;
    std::string line;
    while (std::getline(f, line)) {
        std::vector<double> row;
        std::stringstream ss(line);
        std::string cell;
        while (std::getline(ss, cell, ',')) row.push_back(parse_value(cell));
        if (!row.empty()) m.push_back(row);
    }
    return m;
}

// fem_v2/fem_simulation.cpp:1446-1475: scientific with 6 digits, trailing
// zeros of the mantissa removed, "e+00" dropped.
std::string compress_number(double v)
{
    std::ostringstream oss;
    oss << std::scientific << std::setprecision(6) << v;
    std::string s = oss.str();
    size_t e = s.find_first_of("eE");
    if (e == std::string::npos) return s;
    std::string mant = s.substr(0, e), ex = s.substr(e);
    if (ex == "e+00" || ex == "E+00") ex = "";
    mant.erase(mant.find_last_not_of('0') + 1, std::string::npos);
    if (!mant.empty() && mant.back() == '.') mant.pop_back();
    return mant + ex;
}

void Sim::save_component(int receiver, int component, const char *path) const
{
    EMS_CHECK_ARG(path && *path, "file name required");
    EMS_CHECK_ARG(receiver >= 0 && receiver < nobs, "receiver index out of range");
    EMS_CHECK_ARG(component >= 0 && component < 3, "component must be 0 (x), 1 (y) or 2 (z)");
    std::ofstream f(path);
    if (!f.is_open()) throw Error{EMS_ERR_IO, std::string("cannot open ") + path};
    const int off = ncols == 4 ? 1 : 0;   // FEM tables: t, Ex, Ey, Ez; FDTD: Ex, Ey, Ez
    f << std::setprecision(15) << std::scientific << "t,u" << std::endl;
    for (int j = 0; j < nsamp; ++j)
        f << sample_time(j) << "," << traces[((size_t)receiver * nsamp + j) * ncols + off + component] << std::endl;
}

}  // namespace ems
