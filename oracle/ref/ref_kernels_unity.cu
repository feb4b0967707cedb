// One translation unit with the reference's kernel sources (included from the reference
// checkout by build_ref_kernels.sh, never copied) and a few helper kernels of ours that need
// the reference's own types.  Device code only: compiled with -cubin and loaded by the runner.
#include "coredynamics.cu"
#include "discrete_input_convol.cu"
#include "condShape.cu"
#include "util/cuda_util.cu"

// ConductanceShape as the reference's constructor builds it (src/condShape.h:13-26), written
// byte for byte to out, so that the runner can pass it by value; out[0..3] = sizeof first.
extern "C" __global__ void refh_make_cond(const float *rise, const float *decay, unsigned ng, unsigned char *out) {
    ConductanceShape c(const_cast<float *>(rise), const_cast<float *>(decay), ng);
    const unsigned n = sizeof(ConductanceShape);
    *reinterpret_cast<unsigned *>(out) = n;
    const unsigned char *b = reinterpret_cast<const unsigned char *>(&c);
    for (unsigned i = 0; i < n; i++) out[4 + i] = b[i];
}

// sizeof of the by-value structs the V1 kernels take (learning = 0 passes them zeroed).
extern "C" __global__ void refh_sizes(unsigned *out) {
    out[0] = sizeof(ConductanceShape);
    out[1] = sizeof(LearnVarShapeFF_E_pre);
    out[2] = sizeof(LearnVarShapeFF_I_pre);
    out[3] = sizeof(LearnVarShapeFF_E_post);
    out[4] = sizeof(LearnVarShapeFF_I_post);
    out[5] = sizeof(LearnVarShapeE);
    out[6] = sizeof(LearnVarShapeQ);
    out[7] = sizeof(curandStateMRG32k3a);
    out[8] = sizeof(Spatial_component);
    out[9] = sizeof(Temporal_component);
    out[10] = sizeof(Static_nonlinear);
}
