// Tensor-core (tcgen05) application of dense 6-wire complex64 blocks
// (kernels_tc.cu).
#pragma once

#include "plgb_common.cuh"

namespace plgb {

// Tile geometry of a 6-wire block on an n-qubit register: the 12 local bits
// (block bits and the six lowest other bits) in ascending order, and for
// each local index bit q which member bit (ibit) or group bit (gbit) it is.
struct TcGeom {
    signed char ibit[12];
    signed char gbit[12];
    int lbit[12];
    int glob[64];
    int nglob;
    u64 ntiles;
    unsigned short jj_of_i[64];
    unsigned short jj_of_g[64];
};

// false when the register is too small (fewer than 12 qubits) or the bits
// are not six distinct positions below n; bits6[0] = the matrix's most
// significant local bit (its first wire)
bool tc_geom_for(int n, const int *bits6, TcGeom &g);
// the shared-memory image of a row-major 64 x 64 complex64 matrix: its real
// form split into three BF16 parts (h, m, l) in the MMA operand layout
size_t tc_a_image_bytes();
void tc_build_a_image(const cx<float> *U, unsigned short *img);
// sv <- U on every group of the six bits (img: device copy of the image;
// err: device word set to 1 when a CTA gave up waiting for its MMAs)
void launch_dense6_tc(cudaStream_t s, cx<float> *sv, const TcGeom &geom, const unsigned short *a_img, int *err);

// whether complex64 dense 6-wire gates take the tensor-core kernel
bool tc_dense_enabled();
bool set_tc_dense_enabled(bool on);

} // namespace plgb
