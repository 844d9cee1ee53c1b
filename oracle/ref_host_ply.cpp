// The reference's PLY loader and scene transform, for golden fixtures -- TEST
// INFRASTRUCTURE.
//
// loadPly_torch and computeCov3D (csrc/pybind.cpp:22-120) live in an
// anonymous namespace of the reference's bindings, so this translation unit
// includes that source file where it lies (the include path is given by
// oracle/ref_host.py) and calls loadPly_torch directly: it parses the binary
// PLY, reorders the SH coefficients, applies sigmoid / exp / quaternion
// normalisation and forms the 3D covariance on the CPU.  Built and run on the
// host only; nothing of the reference is copied into this repository.
#include "pybind.cpp"

// Returns the vertex count (at most `capacity` are copied), or -1 on error.
extern "C" int ref_load_ply(const char* path, int capacity, float* pos, float* shs, float* opacity, float* cov3d)
{
    try {
        auto t = polysplat::loadPly_torch(std::string(path));
        const int n = std::get<0>(t);
        const int m = n < capacity ? n : capacity;
        std::memcpy(pos, std::get<1>(t).data_ptr<float>(), sizeof(float) * 3 * (size_t)m);
        std::memcpy(shs, std::get<2>(t).data_ptr<float>(), sizeof(float) * 48 * (size_t)m);
        std::memcpy(opacity, std::get<3>(t).data_ptr<float>(), sizeof(float) * (size_t)m);
        std::memcpy(cov3d, std::get<4>(t).data_ptr<float>(), sizeof(float) * 6 * (size_t)m);
        return n;
    } catch (...) {
        return -1;
    }
}
