// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/small_strato.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 7 species (6 variable), 10 reactions, 26 W slots, 29 LU slots, 29 LU products, 13 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_small_strato {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const int r_off[11] = {0, 1, 3, 4, 6, 7, 8, 10, 12, 14, 15};
static __device__ const int r_y[15] = {2, 1, 2, 3, 1, 3, 3, 0, 0, 3, 4, 3, 5, 1, 5};
static __device__ const int f_off[7] = {0, 3, 10, 18, 24, 27, 30};
static __device__ const int f_r[30] = {4, 5, 6, 0, 1, 2, 3, 5, 8, 9, 0, 1, 2, 3, 4, 6, 7, 8, 1, 2, 3, 4, 6, 7, 7, 8, 9, 7, 8, 9};
static __device__ const double f_c[30] = {1.0, -1.0, -1.0, 2.0, -1.0, 1.0, -1.0, 1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 2.0, 1.0, 2.0, 1.0, 1.0, 1.0, -1.0, -1.0, -1.0, -1.0, -1.0, -1.0, 1.0, 1.0, 1.0, -1.0, -1.0};
static __device__ const int d_r[15] = {0, 1, 1, 2, 3, 3, 4, 5, 6, 6, 7, 7, 8, 8, 9};
static __device__ const int d_off[16] = {0, 0, 1, 2, 2, 3, 4, 4, 4, 5, 6, 7, 8, 9, 10, 10};
static __device__ const int d_fac[10] = {2, 1, 3, 1, 3, 0, 3, 4, 1, 5};
static __device__ const double d_lit[15] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
static __device__ const int w_slot[26] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 19, 21, 22, 23, 24, 26, 27, 28};
static __device__ const int w_diag[26] = {1, 0, 0, 1, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 1, 0, 0, 0, 0, 1};
static __device__ const int w_off[27] = {0, 2, 4, 5, 8, 10, 12, 14, 15, 18, 20, 25, 26, 27, 28, 30, 31, 36, 37, 38, 39, 40, 42, 43, 44, 45, 47};
static __device__ const int w_p[47] = {7, 8, 6, 9, 7, 1, 4, 13, 0, 2, 3, 5, 12, 14, 8, 1, 4, 13, 0, 2, 3, 5, 6, 9, 11, 10, 12, 8, 1, 4, 2, 3, 5, 6, 9, 11, 10, 13, 11, 10, 12, 14, 13, 11, 10, 12, 14};
static __device__ const double w_c[47] = {1.0, 1.0, -1.0, 1.0, -1.0, 1.0, 1.0, 1.0, -2.0, 1.0, -1.0, 1.0, 1.0, -1.0, -2.0, 1.0, -2.0, -1.0, 1.0, 1.0, -1.0, -2.0, -1.0, -2.0, -1.0, -1.0, -1.0, 1.0, -1.0, 1.0, -1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, -1.0, 1.0, 1.0, -1.0, -1.0, 1.0, -1.0, -1.0, 1.0, 1.0};
constexpr int NW = 26;
constexpr int N_LU_ZERO = 3;
static __device__ const int lu_zero[3] = {20, 25, 18};
constexpr int LU_STEPS = 13;
constexpr int SV_STEPS = 19;
static __device__ const unsigned long long lu_fs[416] = {
    0x3000000000000ull, 0x3000000000003ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000000000002ull, 0x2000000000007ull, 0x200000000000dull, 0x2000300000008ull, 0x200030000000eull, 0x2000300000013ull, 0x2000300000018ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000100020005ull, 0x1000400080009ull, 0x100010007000aull, 0x100060008000cull, 0x10004000e000full, 0x1000400130014ull, 0x1000400180019ull, 0x10001000d0010ull,
    0x10006000e0012ull, 0x1000600130017ull, 0x100060018001cull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x3000000000009ull, 0x100050008000aull, 0x10005000e0010ull, 0x1000500130015ull, 0x100050018001aull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x200090000000full, 0x2000900000014ull, 0x2000900000019ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000a000f0010ull, 0x1000b000f0011ull, 0x1000c000f0012ull, 0x1000a00140015ull, 0x1000a0019001aull, 0x1000b00140016ull, 0x1000c00140017ull, 0x1000b0019001bull,
    0x1000c0019001cull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x3000000000010ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2001000000015ull, 0x200100000001aull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1001100150016ull, 0x1001200150017ull, 0x10011001a001bull, 0x10012001a001cull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x3000000000016ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x200160000001bull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10017001b001cull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x300000000001cull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
};
static __device__ const unsigned long long sv_fs[608] = {
    0x1000000020001ull, 0x1000000070002ull, 0x10000000d0003ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000100080002ull, 0x10001000e0003ull, 0x1000100130004ull, 0x1000100180005ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10002000f0003ull, 0x1000200140004ull, 0x1000200190005ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000300150004ull, 0x10003001a0005ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10004001b0005ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2001c00000005ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000500170004ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2001600000004ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000400110003ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000500120003ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2001000000003ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10003000a0002ull, 0x1000300010000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10004000b0002ull, 0x2000000000000ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x10005000c0002ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000900000002ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000200040001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000300050001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x1000500060001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x2000300000001ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
    0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull, 0x0ull,
};
static __device__ const int diag[6] = {0, 3, 9, 16, 22, 28};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "small_strato";
  static constexpr int NS = 7;      // species including fixed ones
  static constexpr int NV = 6;      // variable species (solved system)
  static constexpr int NR = 10;      // reactions
  static constexpr int NP = 4;      // runtime parameter slots per cell
  static constexpr int NPH = 4;      // photolysis slots
  static constexpr int NFIX = 1;
  static constexpr int NLU = 29;
  static constexpr int NSTAGE = 3;
  static constexpr bool RUNTIME_ENV = false;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.435866521508459;
  static constexpr double ELO = 3.0;
  static constexpr double SEED = 9.9999999999999995e-07;
  static constexpr double ENV_T = 298.14999999999998;
  static constexpr double ENV_RHO = 2.46e+19;
  static constexpr long long LU_FMA = 29;
  static constexpr long long LU_SCALE = 13;
  static constexpr long long SOLVE_L = 13;
  static constexpr long long SOLVE_U = 10;
  static constexpr long long FUN_FLOPS = 75;
  static constexpr long long JAC_FLOPS = 104;

  __host__ __device__ static constexpr int var_phys(int i) { constexpr int t[6] = {1, 0, 6, 2, 3, 4}; return t[i]; }
  __host__ __device__ static constexpr int fix_phys(int i) { constexpr int t[1] = {5}; return t[i]; }
  __host__ __device__ static constexpr double atol_v(int i) { constexpr double t[6] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0}; return t[i]; }
  __host__ __device__ static constexpr double rtol_v(int i) { constexpr double t[6] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001}; return t[i]; }
  __host__ __device__ static constexpr int lu_prow(int s) { constexpr int t[29] = {1, 1, 0, 0, 0, 0, 0, 6, 6, 6, 6, 6, 6, 2, 2, 2, 2, 2, 2, 3, 3, 3, 3, 3, 4, 4, 4, 4, 4}; return t[s]; }
  __host__ __device__ static constexpr int lu_pcol(int s) { constexpr int t[29] = {1, 2, 1, 0, 6, 2, 4, 1, 0, 6, 2, 3, 4, 1, 0, 6, 2, 3, 4, 0, 6, 2, 3, 4, 0, 6, 2, 3, 4}; return t[s]; }
  static const char* species_name(int s) { static const char* t[7] = {"O", "O1D", "O3", "NO", "NO2", "M", "O2"}; return t[s]; }
  static const char* photolysis_name(int p) { static const char* t[4] = {"J_1", "J_2", "J_3", "J_4"}; return t[p]; }

  // Rate constants of every reaction (reaction index order).  P(n) is the
  // cell's runtime parameter n (photolysis J_n or external Rate slot n),
  // FIX(s) the concentration of fixed species s, T/RHO the cell's
  // temperature and air density.
  template <class PA, class FA, class KO>
  __device__ __forceinline__ static void rate_constants(const PA& P, const FA& FIX, double T, double RHO,
                                                      double RH, double CLW, KO& k) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX;
    k.set(0, P(0));
    k.set(1, 8.0180000000000003e-17);
    k.set(2, P(1));
    k.set(3, 1.576e-15);
    k.set(4, P(2));
    k.set(5, 7.1100000000000005e-11*FIX(5));
    k.set(6, 1.2e-10);
    k.set(7, 6.0620000000000003e-15);
    k.set(8, 1.0690000000000001e-11);
    k.set(9, P(3));
  }

  // Per-cell working storage, in slots of one double: the LU factors, the
  // state y, the stage vectors K_1..K_s, the tendency F, the increment dy and
  // the rate constants of the current host step.
  static constexpr int Y = 29;
  static constexpr int K0 = 35;
  static constexpr int F = 53;
  static constexpr int DY = 59;
  static constexpr int KT = 65;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 75;

  // Mass-action tendencies F(y) of the variable species (logical order):
  // y(i) supplies the state, out(i, F_i) receives the result.
  template <class YA, class KA, class FO>
  __device__ __forceinline__ static void fun(const YA& y, const KA& k, FO&& out) {
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double y3 = y(3);
    const double y4 = y(4);
    const double y5 = y(5);
    const double q0 = k(0) * y2;
    const double q1 = k(1) * y1 * y2;
    const double q2 = k(2) * y3;
    const double q3 = k(3) * y1 * y3;
    const double q4 = k(4) * y3;
    const double q5 = k(5) * y0;
    const double q6 = k(6) * y0 * y3;
    const double q7 = k(7) * y4 * y3;
    const double q8 = k(8) * y5 * y1;
    const double q9 = k(9) * y5;
    out(0, q4 - q5 - q6);
    out(1, 2.0 * q0 - q1 + q2 - q3 + q5 - q8 + q9);
    out(2, fma(2.0, q6, fma(2.0, q3, -q0 - q1 + q2) + q4) + q7 + q8);
    out(3, q1 - q2 - q3 - q4 - q6 - q7);
    out(4, -q7 + q8 + q9);
    out(5, q7 - q8 - q9);
  }

  // W = I/(gamma h) - J(y) into the LU slots that hold W entries.
  template <class YA, class KA, class SA>
  __device__ __forceinline__ static void jac_w(const YA& y, const KA& k, double inv_g_dt, SA& S) {
    (void)inv_g_dt;
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double y3 = y(3);
    const double y4 = y(4);
    const double y5 = y(5);
    const double d0_2 = k(0);
    const double d1_1 = k(1) * y2;
    const double d1_2 = k(1) * y1;
    const double d2_3 = k(2);
    const double d3_1 = k(3) * y3;
    const double d3_3 = k(3) * y1;
    const double d4_3 = k(4);
    const double d5_0 = k(5);
    const double d6_0 = k(6) * y3;
    const double d6_3 = k(6) * y0;
    const double d7_4 = k(7) * y3;
    const double d7_3 = k(7) * y4;
    const double d8_5 = k(8) * y1;
    const double d8_1 = k(8) * y5;
    const double d9_5 = k(9);
    S[0] = inv_g_dt + d5_0 + d6_0;
    S[1] = -d4_3 + d6_3;
    S[2] = -d5_0;
    S[3] = inv_g_dt + d1_1 + d3_1 + d8_1;
    S[4] = -2.0 * d0_2 + d1_2;
    S[5] = -d2_3 + d3_3;
    S[6] = d8_5 - d9_5;
    S[7] = -2.0 * d6_0;
    S[8] = fma(-2.0, d3_1, d1_1) - d8_1;
    S[9] = inv_g_dt + d0_2 + d1_2;
    S[10] = fma(-2.0, d6_3, fma(-2.0, d3_3, -d2_3) - d4_3) - d7_3;
    S[11] = -d7_4;
    S[12] = -d8_5;
    S[13] = d6_0;
    S[14] = -d1_1 + d3_1;
    S[15] = -d1_2;
    S[16] = inv_g_dt + d2_3 + d3_3 + d4_3 + d6_3 + d7_3;
    S[17] = d7_4;
    S[19] = -d8_1;
    S[21] = d7_3;
    S[22] = inv_g_dt + d7_4;
    S[23] = -d8_5 - d9_5;
    S[24] = d8_1;
    S[26] = -d7_3;
    S[27] = -d7_4;
    S[28] = inv_g_dt + d8_5 + d9_5;
  }

  // Physical (row, column) of every W slot, for the dense Jacobian.
  template <class Fn>
  __device__ __forceinline__ static void for_each_w_slot(Fn&& fn) {
    fn(0, 1, 1);
    fn(1, 1, 2);
    fn(2, 0, 1);
    fn(3, 0, 0);
    fn(4, 0, 6);
    fn(5, 0, 2);
    fn(6, 0, 4);
    fn(7, 6, 1);
    fn(8, 6, 0);
    fn(9, 6, 6);
    fn(10, 6, 2);
    fn(11, 6, 3);
    fn(12, 6, 4);
    fn(13, 2, 1);
    fn(14, 2, 0);
    fn(15, 2, 6);
    fn(16, 2, 2);
    fn(17, 2, 3);
    fn(19, 3, 0);
    fn(21, 3, 2);
    fn(22, 3, 3);
    fn(23, 3, 4);
    fn(24, 4, 0);
    fn(26, 4, 2);
    fn(27, 4, 3);
    fn(28, 4, 4);
  }

  // Fixed-species columns of the dense Jacobian: dF_i/dC_f through the
  // rate constants' dependence on fixed species (third bodies).
  template <class PA, class FA, class YA, class Fn>
  __device__ __forceinline__ static void jac_fixed_columns(const PA& P, const FA& FIX, double T, double RHO,
                                                         double RH, double CLW, const YA& y, Fn&& fn) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX; (void)y;
    fn(0, 5, ((7.1100000000000005e-11) * y(0)));
    fn(1, 5, -((7.1100000000000005e-11) * y(0)));
  }

  // In-place row-wise Doolittle LU over the compact slots, in the operation
  // order of the reference plan.  The operands a row reuses (its own L
  // entries for the U part, the pivot column of U for the L part) are read
  // once into registers.  Diagonal slots end up holding 1/U_ii.
  template <class SA>
  __device__ __forceinline__ static bool factor(SA& S) {
    bool ok = true;
    {  // pivot row 0
      const double u0 = S[0];
      ok = ok && (u0 != 0.0);
      const double rd = 1.0 / u0;
      S[0] = rd;
      double v1 = S[1];
      double v2 = S[2];
      double v7 = S[7];
      double v13 = S[13];
      S[2] = v2 * rd;
      S[7] = v7 * rd;
      S[13] = v13 * rd;
    }
    {  // pivot row 1
      const double a2 = S[2];
      const double u3 = S[3];
      ok = ok && (u3 != 0.0);
      const double rd = 1.0 / u3;
      S[3] = rd;
      double v4 = S[4];
      double v5 = S[5];
      double v6 = S[6];
      v5 = fma(-a2, S[1], v5);
      S[5] = v5;
      double v8 = S[8];
      double v14 = S[14];
      double v19 = S[19];
      double v24 = S[24];
      S[8] = v8 * rd;
      S[14] = v14 * rd;
      S[19] = v19 * rd;
      S[24] = v24 * rd;
    }
    {  // pivot row 2
      const double a7 = S[7];
      const double a8 = S[8];
      const double u9 = fma(-a8, S[4], S[9]);
      ok = ok && (u9 != 0.0);
      const double rd = 1.0 / u9;
      S[9] = rd;
      double v10 = S[10];
      double v11 = S[11];
      double v12 = S[12];
      v10 = fma(-a7, S[1], v10);
      v12 = fma(-a8, S[6], v12);
      v10 = fma(-a8, S[5], v10);
      S[10] = v10;
      S[12] = v12;
      const double b4 = S[4];
      double v15 = S[15];
      double v20 = 0.0;
      double v25 = 0.0;
      v15 = fma(-S[14], b4, v15);
      v20 = fma(-S[19], b4, v20);
      v25 = fma(-S[24], b4, v25);
      S[15] = v15 * rd;
      S[20] = v20 * rd;
      S[25] = v25 * rd;
    }
    {  // pivot row 3
      const double a13 = S[13];
      const double a14 = S[14];
      const double a15 = S[15];
      const double u16 = fma(-a15, S[10], fma(-a14, S[5], fma(-a13, S[1], S[16])));
      ok = ok && (u16 != 0.0);
      const double rd = 1.0 / u16;
      S[16] = rd;
      double v17 = S[17];
      double v18 = 0.0;
      v17 = fma(-a15, S[11], v17);
      v18 = fma(-a14, S[6], v18);
      v18 = fma(-a15, S[12], v18);
      S[17] = v17;
      S[18] = v18;
      const double b5 = S[5];
      const double b10 = S[10];
      double v21 = S[21];
      double v26 = S[26];
      v21 = fma(-S[19], b5, v21);
      v26 = fma(-S[24], b5, v26);
      v21 = fma(-S[20], b10, v21);
      v26 = fma(-S[25], b10, v26);
      S[21] = v21 * rd;
      S[26] = v26 * rd;
    }
    {  // pivot row 4
      const double a19 = S[19];
      const double a20 = S[20];
      const double a21 = S[21];
      const double u22 = fma(-a21, S[17], fma(-a20, S[11], S[22]));
      ok = ok && (u22 != 0.0);
      const double rd = 1.0 / u22;
      S[22] = rd;
      double v23 = S[23];
      v23 = fma(-a19, S[6], v23);
      v23 = fma(-a20, S[12], v23);
      v23 = fma(-a21, S[18], v23);
      S[23] = v23;
      const double b11 = S[11];
      const double b17 = S[17];
      double v27 = S[27];
      v27 = fma(-S[25], b11, v27);
      v27 = fma(-S[26], b17, v27);
      S[27] = v27 * rd;
    }
    {  // pivot row 5
      const double a24 = S[24];
      const double a25 = S[25];
      const double a26 = S[26];
      const double a27 = S[27];
      const double u28 = fma(-a27, S[23], fma(-a26, S[18], fma(-a25, S[12], fma(-a24, S[6], S[28]))));
      ok = ok && (u28 != 0.0);
      const double rd = 1.0 / u28;
      S[28] = rd;
    }
    return ok;
  }

  // Solve (LU) x = b in place on slots [base, base + NV): unit-L forward
  // sweep, then the U backward sweep scaled by the stored 1/U_ii.
  template <class SA>
  __device__ __forceinline__ static void solve(SA& S, const int base) {
    const double v0 = S[base + 0];
    const double v1 = fma(-S[2], v0, S[base + 1]);
    const double v2 = fma(-S[8], v1, fma(-S[7], v0, S[base + 2]));
    const double v3 = fma(-S[15], v2, fma(-S[14], v1, fma(-S[13], v0, S[base + 3])));
    const double v4 = fma(-S[21], v3, fma(-S[20], v2, fma(-S[19], v1, S[base + 4])));
    const double v5 = fma(-S[27], v4, fma(-S[26], v3, fma(-S[25], v2, fma(-S[24], v1, S[base + 5]))));
    const double x5 = (v5) * S[28];
    S[base + 5] = x5;
    const double x4 = (fma(-S[23], x5, v4)) * S[22];
    S[base + 4] = x4;
    const double x3 = (fma(-S[18], x5, fma(-S[17], x4, v3))) * S[16];
    S[base + 3] = x3;
    const double x2 = (fma(-S[12], x5, fma(-S[11], x4, fma(-S[10], x3, v2)))) * S[9];
    S[base + 2] = x2;
    const double x1 = (fma(-S[6], x5, fma(-S[5], x3, fma(-S[4], x2, v1)))) * S[3];
    S[base + 1] = x1;
    const double x0 = (fma(-S[1], x3, v0)) * S[0];
    S[base + 0] = x0;
  }

  // One Rosenbrock attempt of size h from the state in S[Y..].  Returns the
  // WRMS error norm and leaves the increment sum_j M_j K_j in S[DY..].
  // Bit 1 of status is set on a zero pivot.
  template <class SA, class KA>
  __device__ __forceinline__ static double attempt(SA& S, const KA& k, double h, int& status) {
    const double inv_g_dt = 1.0 / (GAMMA * h);
    jac_w([&](int i) { return S[Y + i]; }, k, inv_g_dt, S);
    if (!factor(S)) status |= 1;
    fun([&](int i) { return S[Y + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[35 + i] = S[F + i];
    }
    solve(S, 35);
    fun([&](int i) { return S[Y + i] + S[35 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c21 = -1.0156171083877703 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[41 + i] = fma(c21, S[35 + i], S[F + i]);
    }
    solve(S, 41);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[47 + i] = fma(c32, S[41 + i], fma(c31, S[35 + i], S[F + i]));
    }
    solve(S, 47);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[35 + i];
      const double k1 = S[41 + i];
      const double k2 = S[47 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
      err_sq = fma(q, q, err_sq);
    }
    return fmax(sqrt(err_sq / 7.0), 1.0e-10);
  }

  // Step-size factor from the error norm (integrate.j2:324-333).
  __device__ __forceinline__ static double growth(double err) {
    const double fac = 0.9 / cbrt(err);
    return fmax(0.2, fmin(fac, 6.0));
  }

  // ---- warp-cooperative attempt (tables + static warp schedules) ----
  static constexpr int NPART = 15;
  static constexpr int Q = NSLOTS;            // rates q_r, then q_i of the error norm
  static constexpr int D = NSLOTS + 10;     // partial derivatives
  static constexpr int COOP_SLOTS = NSLOTS + 10 + NPART;
  __device__ __forceinline__ static double acc_term(bool first, double acc, double coef, double t) {
    if (first) return coef == 1.0 ? t : (coef == -1.0 ? -t : coef * t);
    return coef == 1.0 ? acc + t : (coef == -1.0 ? acc - t : fma(coef, t, acc));
  }

  // F(y) into S[F..] for the state yv (S[Y..] or the stage state), cooperatively.
  template <class KA>
  __device__ __forceinline__ static void fun_coop(double* S, const double* yv, const KA& k, unsigned lane) {
    namespace T = coop;
    for (int r = lane; r < NR; r += 32) {
      double q = k(r);
      for (int e = T::r_off[r]; e < T::r_off[r + 1]; ++e) q = q * yv[T::r_y[e]];
      S[Q + r] = q;
    }
    __syncwarp();
    for (int i = lane; i < NV; i += 32) {
      double v = 0.0;
      for (int e = T::f_off[i]; e < T::f_off[i + 1]; ++e) v = acc_term(e == T::f_off[i], v, T::f_c[e], S[Q + T::f_r[e]]);
      S[F + i] = v;
    }
    __syncwarp();
  }

  // Run a static warp schedule (emitter/warp_schedule.py) on S: one
  // multiply-add, pivot multiply or reciprocal per lane and step, a warp
  // barrier between steps.  `out`, and `b` of a multiply-add, are offset by
  // base.  The next two steps' words are in flight while one executes.
  // Returns false if a reciprocal met a zero pivot.
  __device__ __forceinline__ static bool run_schedule(double* S, const unsigned long long* __restrict__ T,
                                                     int steps, int base, unsigned lane) {
    bool ok = true;
    unsigned long long cur = __ldg(T + lane);
    unsigned long long nxt = steps > 1 ? __ldg(T + 32 + lane) : 0ull;
    for (int s = 0; s < steps; ++s) {
      const unsigned long long nn = s + 2 < steps ? __ldg(T + (size_t)(s + 2) * 32 + lane) : 0ull;
      const int kind = (int)(cur >> 48) & 3;
      if (kind != 0) {
        const int out = (int)(cur & 0xffffu) + base;
        const int ia = (int)((cur >> 16) & 0xffffu);
        const int ib = (int)((cur >> 32) & 0xffffu) + (kind == 1 ? base : 0);
        const double vo = S[out];
        if (kind == 3) {
          ok = ok && (vo != 0.0);
          S[out] = 1.0 / vo;
        } else {
          // fma(-a, b, o) for a multiply-add; fma(o, b, -0.0) == o * b exactly.
          const double vb = S[ib];
          const double x = kind == 1 ? -S[ia] : vo;
          const double z = kind == 1 ? vo : -0.0;
          S[out] = fma(x, vb, z);
        }
      }
      __syncwarp();
      cur = nxt;
      nxt = nn;
    }
    return ok;
  }

  // Solve (LU) x = b in place on S[base..].
  __device__ __forceinline__ static void solve_coop(double* S, int base, unsigned lane) {
    run_schedule(S, coop::sv_fs, coop::SV_STEPS, base, lane);
  }

  // One attempt by a whole warp on the cell held in shared memory S
  // (NSLOTS + NR + NPART doubles).  Same values as attempt(); the error norm
  // is summed by lane 0 in species order.  Returns err on every lane.
  template <class KA>
  __device__ __forceinline__ static double attempt_coop(double* S, const KA& k, double h, int& status,
                                                       unsigned lane) {
    namespace T = coop;
    const double inv_g_dt = 1.0 / (GAMMA * h);
    // Jacobian partials, then W into the LU slots.
    for (int p = lane; p < NPART; p += 32) {
      double d = k(T::d_r[p]);
      for (int e = T::d_off[p]; e < T::d_off[p + 1]; ++e) {
        const int f = T::d_fac[e];
        d = d * (f < 0 ? T::d_lit[p] : S[Y + f]);
      }
      S[D + p] = d;
    }
    __syncwarp();
    for (int z = lane; z < T::N_LU_ZERO; z += 32) S[T::lu_zero[z]] = 0.0;
    for (int w = lane; w < T::NW; w += 32) {
      bool first = !T::w_diag[w];
      double v = T::w_diag[w] ? inv_g_dt : 0.0;
      for (int e = T::w_off[w]; e < T::w_off[w + 1]; ++e) {
        v = acc_term(first, v, T::w_c[e], S[D + T::w_p[e]]);
        first = false;
      }
      S[T::w_slot[w]] = v;
    }
    __syncwarp();
    // LU by the static warp schedule (fill-in slots were zeroed with W).
    const bool ok = run_schedule(S, T::lu_fs, T::LU_STEPS, 0, lane);
    if (__any_sync(0xffffffffu, !ok)) status |= 1;
    fun_coop(S, S + Y, k, lane);
    for (int i = lane; i < NV; i += 32) S[35 + i] = S[F + i];
    __syncwarp();
    solve_coop(S, 35, lane);
    // Stage state into the DY slots (free until the error block).
    for (int i = lane; i < NV; i += 32) S[DY + i] = S[Y + i] + S[35 + i];
    __syncwarp();
    fun_coop(S, S + DY, k, lane);
    const double c21 = -1.0156171083877703 / h;
    for (int i = lane; i < NV; i += 32) S[41 + i] = fma(c21, S[35 + i], S[F + i]);
    __syncwarp();
    solve_coop(S, 41, lane);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    for (int i = lane; i < NV; i += 32) S[47 + i] = fma(c32, S[41 + i], fma(c31, S[35 + i], S[F + i]));
    __syncwarp();
    solve_coop(S, 47, lane);
    // Increment, and q_i^2 of the error norm into the rate slots.
    for (int i = lane; i < NV; i += 32) {
      const double k0 = S[35 + i];
      const double k1 = S[41 + i];
      const double k2 = S[47 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      S[Q + i] = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
    }
    __syncwarp();
    double err = 0.0;
    if (lane == 0) {
      double err_sq = 0.0;
      for (int i = 0; i < NV; ++i) err_sq = fma(S[Q + i], S[Q + i], err_sq);
      err = fmax(sqrt(err_sq / 7.0), 1.0e-10);
    }
    return __shfl_sync(0xffffffffu, err, 0);
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 75;      // dL/dy
  static constexpr int KBAR = 81;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 99;    // adjoint of the pending stage tendency
  static constexpr int KB = 105;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 115;
  // Solve W^T x = b in place on [base, base + NV) with the stored LU of W.
  template <class SA>
  __device__ __noinline__ static void solve_t(SA& S, const int base) {
    const double z0 = (S[base + 0]) * S[0];
    const double z1 = (S[base + 1]) * S[3];
    const double z2 = (fma(-S[4], z1, S[base + 2])) * S[9];
    const double z3 = (fma(-S[10], z2, fma(-S[5], z1, fma(-S[1], z0, S[base + 3])))) * S[16];
    const double z4 = (fma(-S[17], z3, fma(-S[11], z2, S[base + 4]))) * S[22];
    const double z5 = (fma(-S[23], z4, fma(-S[18], z3, fma(-S[12], z2, fma(-S[6], z1, S[base + 5]))))) * S[28];
    const double x5 = z5;
    S[base + 5] = x5;
    const double x4 = fma(-S[27], x5, z4);
    S[base + 4] = x4;
    const double x3 = fma(-S[26], x5, fma(-S[21], x4, z3));
    S[base + 3] = x3;
    const double x2 = fma(-S[25], x5, fma(-S[20], x4, fma(-S[15], x3, z2)));
    S[base + 2] = x2;
    const double x1 = fma(-S[24], x5, fma(-S[19], x4, fma(-S[14], x3, fma(-S[8], x2, z1))));
    S[base + 1] = x1;
    const double x0 = fma(-S[13], x3, fma(-S[7], x2, fma(-S[2], x1, z0)));
    S[base + 0] = x0;
  }

  // u^T J(y) v terms of stage i: y in S[Y..], u in S[ub..], v = K_i in S[vb..].
  template <class SA, class KA>
  __device__ __noinline__ static void adj_wterm(SA& S, const KA& k, const int ub, const int vb) {
    auto u = [&](int i) { return S[ub + i]; };
    const double y0 = S[Y + 0];
    const double v0 = S[vb + 0];
    const double y1 = S[Y + 1];
    const double v1 = S[vb + 1];
    const double y2 = S[Y + 2];
    const double v2 = S[vb + 2];
    const double y3 = S[Y + 3];
    const double v3 = S[vb + 3];
    const double y4 = S[Y + 4];
    const double v4 = S[vb + 4];
    const double y5 = S[Y + 5];
    const double v5 = S[vb + 5];
    { const double s = fma(2.0, u(1), -u(2));
      S[KB + 0] = fma(s, v2, S[KB + 0]);
      const double ks = k(0) * s;
    }
    { const double s = -u(1) - u(2) + u(3);
      S[KB + 1] = fma(s, (y2) * v1 + (y1) * v2, S[KB + 1]);
      const double ks = k(1) * s;
      S[LAM + 1] = fma(ks, v2, S[LAM + 1]);
      S[LAM + 2] = fma(ks, v1, S[LAM + 2]);
    }
    { const double s = -u(3) + u(1) + u(2);
      S[KB + 2] = fma(s, v3, S[KB + 2]);
      const double ks = k(2) * s;
    }
    { const double s = fma(2.0, u(2), -u(1) - u(3));
      S[KB + 3] = fma(s, (y3) * v1 + (y1) * v3, S[KB + 3]);
      const double ks = k(3) * s;
      S[LAM + 1] = fma(ks, v3, S[LAM + 1]);
      S[LAM + 3] = fma(ks, v1, S[LAM + 3]);
    }
    { const double s = -u(3) + u(0) + u(2);
      S[KB + 4] = fma(s, v3, S[KB + 4]);
      const double ks = k(4) * s;
    }
    { const double s = -u(0) + u(1);
      S[KB + 5] = fma(s, v0, S[KB + 5]);
      const double ks = k(5) * s;
    }
    { const double s = fma(2.0, u(2), -u(0) - u(3));
      S[KB + 6] = fma(s, (y3) * v0 + (y0) * v3, S[KB + 6]);
      const double ks = k(6) * s;
      S[LAM + 0] = fma(ks, v3, S[LAM + 0]);
      S[LAM + 3] = fma(ks, v0, S[LAM + 3]);
    }
    { const double s = -u(4) - u(3) + u(5) + u(2);
      S[KB + 7] = fma(s, (y4) * v3 + (y3) * v4, S[KB + 7]);
      const double ks = k(7) * s;
      S[LAM + 3] = fma(ks, v4, S[LAM + 3]);
      S[LAM + 4] = fma(ks, v3, S[LAM + 4]);
    }
    { const double s = -u(5) - u(1) + u(4) + u(2);
      S[KB + 8] = fma(s, (y5) * v1 + (y1) * v5, S[KB + 8]);
      const double ks = k(8) * s;
      S[LAM + 1] = fma(ks, v5, S[LAM + 1]);
      S[LAM + 5] = fma(ks, v1, S[LAM + 5]);
    }
    { const double s = -u(5) + u(4) + u(1);
      S[KB + 9] = fma(s, v5, S[KB + 9]);
      const double ks = k(9) * s;
    }
  }

  // Adjoint of F_i = f(Y_i): Ybar = J(Y_i)^T Fbar, kbar += m_r(Y_i) (net_r.Fbar).
  // yv(i) supplies Y_i, ybar(j, x) receives Ybar_j.
  template <class SA, class KA, class YA, class OUT>
  __device__ __forceinline__ static void adj_fterm(SA& S, const KA& k, const YA& yv, OUT&& ybar) {
    auto fb = [&](int i) { return S[FBAR + i]; };
    const double y0 = yv(0);
    const double y1 = yv(1);
    const double y2 = yv(2);
    const double y3 = yv(3);
    const double y4 = yv(4);
    const double y5 = yv(5);
    const double s0 = fma(2.0, fb(1), -fb(2));
    S[KB + 0] = fma(s0, y2, S[KB + 0]);
    const double s1 = -fb(1) - fb(2) + fb(3);
    S[KB + 1] = fma(s1, y1 * y2, S[KB + 1]);
    const double s2 = -fb(3) + fb(1) + fb(2);
    S[KB + 2] = fma(s2, y3, S[KB + 2]);
    const double s3 = fma(2.0, fb(2), -fb(1) - fb(3));
    S[KB + 3] = fma(s3, y1 * y3, S[KB + 3]);
    const double s4 = -fb(3) + fb(0) + fb(2);
    S[KB + 4] = fma(s4, y3, S[KB + 4]);
    const double s5 = -fb(0) + fb(1);
    S[KB + 5] = fma(s5, y0, S[KB + 5]);
    const double s6 = fma(2.0, fb(2), -fb(0) - fb(3));
    S[KB + 6] = fma(s6, y0 * y3, S[KB + 6]);
    const double s7 = -fb(4) - fb(3) + fb(5) + fb(2);
    S[KB + 7] = fma(s7, y3 * y4, S[KB + 7]);
    const double s8 = -fb(5) - fb(1) + fb(4) + fb(2);
    S[KB + 8] = fma(s8, y1 * y5, S[KB + 8]);
    const double s9 = -fb(5) + fb(4) + fb(1);
    S[KB + 9] = fma(s9, y5, S[KB + 9]);
    ybar(0, k(5) * s5 + k(6) * s6 * y3);
    ybar(1, k(1) * s1 * y2 + k(3) * s3 * y3 + k(8) * s8 * y5);
    ybar(2, k(0) * s0 + k(1) * s1 * y1);
    ybar(3, k(2) * s2 + k(3) * s3 * y1 + k(4) * s4 + k(6) * s6 * y0 + k(7) * s7 * y4);
    ybar(4, k(7) * s7 * y3);
    ybar(5, k(8) * s8 * y1 + k(9) * s9);
  }

  // Reverse of one accepted step of size h.  Requires the values attempt()
  // left in S for this step (LU, K_i) and y_n in S[Y..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 6 + j] = 6.1697947043828245 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 12 + j] = -0.42772256543218573 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 12);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 12, 47);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 12 + j];
    { const double cc = 4.0759956452537702 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 12 + q], S[KBAR + 0 + q]); }
    { const double cc = 9.20767942983308 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 6 + q] = fma(cc, S[KBAR + 12 + q], S[KBAR + 6 + q]); }
    // stage 2
    solve_t(S, KBAR + 6);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 6, 41);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 6 + j];
    { const double cc = -1.0156171083877703 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 0 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + S[35 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(1.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 1
    solve_t(S, KBAR + 0);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 0, 35);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 0 + j];
    adj_fterm(S, k, [&](int q) { return S[Y + q]; },
              [&](int j, double x) { S[LAM + j] += x; });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
  }
};

}  // namespace mkpp_small_strato
