// Host (double) entry points over polysplat_gb300/csrc/adjoint.h, built by
// tests/test_adjoint.py to check the preprocess adjoint against central
// differences of the same forward.
#include "../polysplat_gb300/csrc/adjoint.h"

using namespace gsr_adj;

static Cam<double> make_cam(const double* view, const double* proj, const double* campos, const double* f4,
                            const int* wh)
{
    Cam<double> c;
    for (int i = 0; i < 16; i++) {
        c.view[i] = view[i];
        c.proj[i] = proj[i];
    }
    for (int i = 0; i < 3; i++) c.campos[i] = campos[i];
    c.fx = f4[0];
    c.fy = f4[1];
    c.tanx = f4[2];
    c.tany = f4[3];
    c.W = wh[0];
    c.H = wh[1];
    return c;
}

// params: m[3] ls[3] q[4] logit sh[48] (59 values); out: xy[2] con[4] rgb[3] depth (10 values)
extern "C" void adj_forward(const double* params, const double* view, const double* proj, const double* campos,
                            const double* f4, const int* wh, double* out, int* flags)
{
    Cam<double> c = make_cam(view, proj, campos, f4, wh);
    Fwd<double> f;
    Tape<double> tp;
    forward(params, params + 3, params + 6, params[10], params + 11, c, f, tp);
    for (int i = 0; i < 2; i++) out[i] = f.xy[i];
    for (int i = 0; i < 4; i++) out[2 + i] = f.con[i];
    for (int i = 0; i < 3; i++) out[6 + i] = f.rgb[i];
    out[9] = f.depth;
    flags[0] = tp.clamp_x;
    flags[1] = tp.clamp_y;
    for (int i = 0; i < 3; i++) flags[2 + i] = tp.clamp_rgb[i];
}

// g: dL/d(xy[2], con[4], rgb[3]); grad: 59 values in the params layout
extern "C" void adj_backward(const double* params, const double* view, const double* proj, const double* campos,
                             const double* f4, const int* wh, const double* g, double* grad)
{
    Cam<double> c = make_cam(view, proj, campos, f4, wh);
    Fwd<double> f;
    Tape<double> tp;
    forward(params, params + 3, params + 6, params[10], params + 11, c, f, tp);
    double glogit = 0;
    backward(params, params + 11, c, tp, g, g + 2, g + 6, grad, grad + 3, grad + 6, glogit, grad + 11);
    grad[10] = glogit;
}
