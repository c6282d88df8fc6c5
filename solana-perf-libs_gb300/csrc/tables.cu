// Init kernels deriving the curve constants and basepoint tables on the
// device (see tables.cuh for the layouts).  Runs once per device.
#include <cuda_runtime.h>
#include "tables.cuh"

namespace {

__device__ void to_affine_niels(ge_niels& n, const ge_p3& p, const fe& d2) {
    fe zi, x, y, t;
    fe_invert(zi, p.Z);
    fe_mul(x, p.X, zi);
    fe_mul(y, p.Y, zi);
    fe_canon(x, x);
    fe_canon(y, y);
    fe_add(t, y, x);
    fe_canon(n.YpX, t);
    fe_sub(t, y, x);
    fe_canon(n.YmX, t);
    fe_mul(t, x, y);
    fe_mul(t, t, d2);
    fe_canon(n.XY2d, t);
}

__device__ void p3_add(ge_p3& r, const ge_p3& p, const ge_p3& q, const fe& d2) {
    ge_cached c;
    ge_p3_to_cached(c, q, d2);
    ge_done t;
    ge_add_cached(t, p, c, false);
    ge_to_p3(r, t);
}

__device__ void p3_dbl(ge_p3& r, const ge_p3& p) {
    ge_done t;
    ge_dbl(t, p.X, p.Y, p.Z);
    ge_to_p3(r, t);
}

// One thread: constants and the base point.
__global__ void init_consts_kernel(CurveTables* T) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    fe n, dd, t;
    fe_set(n, 121665);
    fe_neg(n, n);
    fe_set(dd, 121666);
    fe_invert(dd, dd);
    fe_mul(t, n, dd);
    fe_canon(T->K.d, t);
    fe_add(t, T->K.d, T->K.d);
    fe_canon(T->K.d2, t);
    // sqrt(-1) = 2^((p-1)/4), (p-1)/4 = 8 * (2^250 - 1) + 3
    fe two, eight, e250, z11;
    fe_set(two, 2);
    fe_set(eight, 8);
    fe_pow2_250_1(e250, z11, two);
    fe_sqn(t, e250, 3);
    fe_mul(t, t, eight);
    fe_canon(T->K.sqrtm1, t);
    // B: y = 4/5, x even
    fe y, five;
    fe_set(five, 5);
    fe_invert(five, five);
    fe_set(y, 4);
    fe_mul(y, y, five);
    fe_canon(y, y);
    uint32_t w[8];
#pragma unroll
    for (int i = 0; i < 8; i++) w[i] = y.v[i];
    fe x, yy;
    ge_decode(x, yy, w, T->K);
    fe_canon(T->B_x, x);
    fe_canon(T->B_y, yy);
}

__device__ void base_point(ge_p3& B, const CurveTables* T) {
    B.X = T->B_x;
    B.Y = T->B_y;
    fe_set(B.Z, 1);
    fe_mul(B.T, T->B_x, T->B_y);
}

// Verify table: k*B, k = 0..128.  Thread k computes its own entry.
__global__ void init_vb_kernel(CurveTables* T) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= VB_ENTRIES) return;
    ge_niels e;
    if (k == 0) {
        fe_set(e.YpX, 1);
        fe_set(e.YmX, 1);
        fe_set(e.XY2d, 0);
    } else {
        ge_p3 B, acc;
        base_point(B, T);
        acc = B;
        // double-and-add over the bits of k below the top one
        int top = 31 - __clz(k);
        for (int bit = top - 1; bit >= 0; bit--) {
            p3_dbl(acc, acc);
            if ((k >> bit) & 1) p3_add(acc, acc, B, T->K.d2);
        }
        to_affine_niels(e, acc, T->K.d2);
    }
#pragma unroll
    for (int w = 0; w < 8; w++) {
        T->vb[(0 + w) * VB_ENTRIES + k] = e.YpX.v[w];
        T->vb[(8 + w) * VB_ENTRIES + k] = e.YmX.v[w];
        T->vb[(16 + w) * VB_ENTRIES + k] = e.XY2d.v[w];
    }
}

// Signing comb: (j+1) * 16^i * B.  Thread (i, j).
__global__ void init_comb_kernel(CurveTables* T) {
    int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= COMB_WINDOWS * COMB_ENTRIES) return;
    int i = id / COMB_ENTRIES, j = id % COMB_ENTRIES;
    ge_p3 P;
    base_point(P, T);
    for (int k = 0; k < 4 * i; k++) p3_dbl(P, P);   // 16^i B
    ge_p3 acc = P;
    for (int k = 0; k < j; k++) p3_add(acc, acc, P, T->K.d2);
    to_affine_niels(T->comb[i][j], acc, T->K.d2);
}

}  // namespace

cudaError_t crypt_tables_create(CurveTables** out, cudaStream_t stream) {
    *out = nullptr;
    CurveTables* T = nullptr;
    cudaError_t e = cudaMalloc(&T, sizeof(CurveTables));
    if (e != cudaSuccess) return e;
    init_consts_kernel<<<1, 32, 0, stream>>>(T);
    init_vb_kernel<<<(VB_ENTRIES + 63) / 64, 64, 0, stream>>>(T);
    init_comb_kernel<<<(COMB_WINDOWS * COMB_ENTRIES + 63) / 64, 64, 0, stream>>>(T);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        cudaFree(T);
        return e;
    }
    *out = T;
    return cudaSuccess;
}
