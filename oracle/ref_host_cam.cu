// The reference's host-side camera matrices, for golden fixtures -- TEST
// INFRASTRUCTURE.
//
// getViewMatrix / getProjectionMatrix (csrc/cuda_rasterizer/preprocess.cu:
// 643-671) live in an anonymous namespace of the reference's preprocess.cu,
// so this translation unit includes that source file where it lies (the
// include path is given by oracle/ref_host.py) and calls them directly.  The
// camera-to-world rotation is turned into a glm::mat3 exactly as the
// reference's bindings do (csrc/pybind.cpp:141-143: JSON row r becomes
// column r).  Built and run on the host only; nothing of the reference is
// copied into this repository.
#include "cuda_rasterizer/preprocess.cu"

extern "C" void ref_camera_matrices(int width, int height, const float* pos, const float* rot, float focal_x,
                                    float focal_y, float z_far, float z_near, float* view16, float* proj16)
{
    const glm::vec3 p({pos[0], pos[1], pos[2]});
    const glm::mat3 r({{rot[0], rot[1], rot[2]}, {rot[3], rot[4], rot[5]}, {rot[6], rot[7], rot[8]}});
    const glm::mat4 v = polysplat::getViewMatrix(p, r);
    const glm::mat4 m = polysplat::getProjectionMatrix(width, height, p, r, focal_x, focal_y, z_far, z_near);
    for (int c = 0; c < 4; c++)
        for (int k = 0; k < 4; k++) {
            view16[4 * c + k] = v[c][k];
            proj16[4 * c + k] = m[c][k];
        }
}
