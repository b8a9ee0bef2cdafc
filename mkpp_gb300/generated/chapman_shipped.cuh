// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/chapman_shipped.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 4 species (3 variable), 4 reactions, 9 W slots, 9 LU slots, 5 LU products, 3 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_chapman_shipped {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const double const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, -2.0, 2.0};
static __device__ const int stage_step[4] = {0, 16, 32, 43};
static __device__ const unsigned long long sched[1376] = {
    0x29002b001b0023ull, 0x29000b001c0024ull, 0x29000a001c0025ull, 0x29002b001d0026ull, 0x290009001e0027ull, 0x29000a001e0028ull, 0x29000b001b001full, 0x29000a001c0020ull,
    0x290009001d0021ull, 0x29000a001e0022ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002b00260000ull, 0x29002b80240001ull, 0x29002b80250002ull, 0x29002b80260003ull, 0x2c002b00240004ull, 0x29003000230005ull, 0x29002b80260006ull, 0x29002b00240007ull,
    0x2c002b00230008ull, 0x29000b00200020ull, 0x29000900220022ull, 0x290031001f0016ull, 0x29002b801f0017ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b00280000ull, 0x1002b00270001ull, 0x3002b00280003ull, 0x4002b00270004ull, 0x5002b00250005ull, 0x6002800300006ull, 0x7002700300007ull, 0x8002b00250008ull,
    0x29002b00200015ull, 0x16002b80200016ull, 0x17002b80200017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000000ull, 0x15002b80210015ull, 0x16002b00210016ull, 0x17002b00210017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000000030003ull, 0x29000000060006ull, 0x15002b80220015ull, 0x16002b80220016ull, 0x17002200310017ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4000180030004ull, 0x5000280030005ull, 0x7000180060007ull, 0x8000280060008ull, 0x29002b0015000cull, 0x29002b0016000dull, 0x29002b0017000eull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000004ull, 0xd000c8003000dull, 0xe000c8006000eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000400070007ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000580070008ull, 0xe000d8007000eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000008ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x290008000e000eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xd000e8005000dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x290004000d000dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xc000d8001000cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xc000e8002000cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x290000000c000cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x9002b000c0018ull, 0xa002b000d0019ull, 0xb002b000e001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29001a001b001full, 0x290019001c0020ull, 0x290018001d0021ull, 0x290019001e0022ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29001a00200020ull, 0x29001800220022ull, 0x290031001f0016ull, 0x29002b801f0017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29002b00200015ull, 0x16002b80200016ull, 0x17002b80200017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15002b80210015ull, 0x16002b00210016ull, 0x17002b00210017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15002b80220015ull, 0x16002b80220016ull, 0x17002200310017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29002b0015000full, 0x29002b00160010ull, 0x29002b00170011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xf000c002d000full, 0x10000d002d0010ull, 0x11000e002d0011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x10000f80030010ull, 0x11000f80060011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x11001080070011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000800110011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x10001180050010ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000400100010ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xf00108001000full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xf00118002000full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x290000000f000full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29002b00150012ull, 0x29002b00160013ull, 0x29002b00170014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12000c002e0012ull, 0x13000d002e0013ull, 0x14000e002e0014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12000f002f0012ull, 0x130010002f0013ull, 0x140011002f0014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x13001280030013ull, 0x14001280060014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x14001380070014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000800140014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x13001480050013ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000400130013ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12001380010012ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12001480020012ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x29000000120012ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
};
constexpr int TLM_OPS = 291;
static __device__ const double tlm_const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 2.0, 6.1697947043828245, -0.42772256543218573};
static __device__ const unsigned long long tlm_prog[291] = {
    0x54005400540042ull, 0x54005400540043ull, 0x54005400540044ull, 0x5400540054004bull, 0x5300550034004dull, 0x4b0055004d004bull, 0x53004b001b004bull, 0x530055000b004cull,
    0x4b004c0035004bull, 0x440055804b0044ull, 0x43004b00590043ull, 0x5400540054004bull, 0x530033000b004dull, 0x4b0055004d004bull, 0x530034000a004dull, 0x4b0055004d004bull,
    0x53004b001c004bull, 0x53000b000a004cull, 0x4b004c0036004bull, 0x430055804b0043ull, 0x440055804b0044ull, 0x420055004b0042ull, 0x5400540054004bull, 0x5300550032004dull,
    0x4b0055004d004bull, 0x53004b001d004bull, 0x5300550009004cull, 0x4b004c0037004bull, 0x420055804b0042ull, 0x430055004b0043ull, 0x440055004b0044ull, 0x5400540054004bull,
    0x530032000a004dull, 0x4b0055004d004bull, 0x5300330009004dull, 0x4b0055004d004bull, 0x53004b001e004bull, 0x53000a0009004cull, 0x4b004c0038004bull, 0x430055804b0043ull,
    0x420055804b0042ull, 0x44004b00590044ull, 0x53005500420039ull, 0x5300550043003aull, 0x5300550044003bull, 0x5400540054004bull, 0x530055000e004dull, 0x4b0055004d004bull,
    0x53004b0035004bull, 0x5400540054004cull, 0x4b004c001b004bull, 0x3b0055804b003bull, 0x3a004b0059003aull, 0x5400540054004bull, 0x53000d000b004dull, 0x4b0055004d004bull,
    0x53000e000a004dull, 0x4b0055004d004bull, 0x53004b0036004bull, 0x5400540054004cull, 0x530034000d004dull, 0x4c0055004d004cull, 0x530033000e004dull, 0x4c0055004d004cull,
    0x4b004c001c004bull, 0x3a0055804b003aull, 0x3b0055804b003bull, 0x390055004b0039ull, 0x5400540054004bull, 0x530055000c004dull, 0x4b0055004d004bull, 0x53004b0037004bull,
    0x5400540054004cull, 0x4b004c001d004bull, 0x390055804b0039ull, 0x3a0055004b003aull, 0x3b0055004b003bull, 0x5400540054004bull, 0x53000c000a004dull, 0x4b0055004d004bull,
    0x53000d0009004dull, 0x4b0055004d004bull, 0x53004b0038004bull, 0x5400540054004cull, 0x530033000c004dull, 0x4c0055004d004cull, 0x530032000d004dull, 0x4c0055004d004cull,
    0x4b004c001e004bull, 0x3a0055804b003aull, 0x390055804b0039ull, 0x3b004b0059003bull, 0x3a00398003003aull, 0x3b00398006003bull, 0x3b003a8007003bull, 0x530008003b003bull,
    0x3a003b8005003aull, 0x530004003a003aull, 0x39003a80010039ull, 0x39003b80020039ull, 0x53000000390039ull, 0x53005500090045ull, 0x53005500320048ull, 0x450055000c0045ull,
    0x48005500390048ull, 0x530055000a0046ull, 0x53005500330049ull, 0x460055000d0046ull, 0x490055003a0049ull, 0x530055000b0047ull, 0x5300550034004aull, 0x470055000e0047ull,
    0x4a0055003b004aull, 0x54005400540042ull, 0x54005400540043ull, 0x54005400540044ull, 0x5400540054004bull, 0x530055004a004dull, 0x4b0055004d004bull, 0x53004b001b004bull,
    0x5300550047004cull, 0x4b004c0035004bull, 0x440055804b0044ull, 0x43004b00590043ull, 0x5400540054004bull, 0x5300490047004dull, 0x4b0055004d004bull, 0x53004a0046004dull,
    0x4b0055004d004bull, 0x53004b001c004bull, 0x5300470046004cull, 0x4b004c0036004bull, 0x430055804b0043ull, 0x440055804b0044ull, 0x420055004b0042ull, 0x5400540054004bull,
    0x5300550048004dull, 0x4b0055004d004bull, 0x53004b001d004bull, 0x5300550045004cull, 0x4b004c0037004bull, 0x420055804b0042ull, 0x430055004b0043ull, 0x440055004b0044ull,
    0x5400540054004bull, 0x5300480046004dull, 0x4b0055004d004bull, 0x5300490045004dull, 0x4b0055004d004bull, 0x53004b001e004bull, 0x5300460045004cull, 0x4b004c0038004bull,
    0x430055804b0043ull, 0x420055804b0042ull, 0x44004b00590044ull, 0x5300550042003cull, 0x3c00390056003cull, 0x5300550043003dull, 0x3d003a0056003dull, 0x5300550044003eull,
    0x3e003b0056003eull, 0x5400540054004bull, 0x5300550011004dull, 0x4b0055004d004bull, 0x53004b0035004bull, 0x5400540054004cull, 0x4b004c001b004bull, 0x3e0055804b003eull,
    0x3d004b0059003dull, 0x5400540054004bull, 0x530010000b004dull, 0x4b0055004d004bull, 0x530011000a004dull, 0x4b0055004d004bull, 0x53004b0036004bull, 0x5400540054004cull,
    0x5300340010004dull, 0x4c0055004d004cull, 0x5300330011004dull, 0x4c0055004d004cull, 0x4b004c001c004bull, 0x3d0055804b003dull, 0x3e0055804b003eull, 0x3c0055004b003cull,
    0x5400540054004bull, 0x530055000f004dull, 0x4b0055004d004bull, 0x53004b0037004bull, 0x5400540054004cull, 0x4b004c001d004bull, 0x3c0055804b003cull, 0x3d0055004b003dull,
    0x3e0055004b003eull, 0x5400540054004bull, 0x53000f000a004dull, 0x4b0055004d004bull, 0x5300100009004dull, 0x4b0055004d004bull, 0x53004b0038004bull, 0x5400540054004cull,
    0x530033000f004dull, 0x4c0055004d004cull, 0x5300320010004dull, 0x4c0055004d004cull, 0x4b004c001e004bull, 0x3d0055804b003dull, 0x3c0055804b003cull, 0x3e004b0059003eull,
    0x3d003c8003003dull, 0x3e003c8006003eull, 0x3e003d8007003eull, 0x530008003e003eull, 0x3d003e8005003dull, 0x530004003d003dull, 0x3c003d8001003cull, 0x3c003e8002003cull,
    0x530000003c003cull, 0x5300550042003full, 0x3f00390057003full, 0x3f003c0058003full, 0x53005500430040ull, 0x40003a00570040ull, 0x40003d00580040ull, 0x53005500440041ull,
    0x41003b00570041ull, 0x41003e00580041ull, 0x5400540054004bull, 0x5300550014004dull, 0x4b0055004d004bull, 0x53004b0035004bull, 0x5400540054004cull, 0x4b004c001b004bull,
    0x410055804b0041ull, 0x40004b00590040ull, 0x5400540054004bull, 0x530013000b004dull, 0x4b0055004d004bull, 0x530014000a004dull, 0x4b0055004d004bull, 0x53004b0036004bull,
    0x5400540054004cull, 0x5300340013004dull, 0x4c0055004d004cull, 0x5300330014004dull, 0x4c0055004d004cull, 0x4b004c001c004bull, 0x400055804b0040ull, 0x410055804b0041ull,
    0x3f0055004b003full, 0x5400540054004bull, 0x5300550012004dull, 0x4b0055004d004bull, 0x53004b0037004bull, 0x5400540054004cull, 0x4b004c001d004bull, 0x3f0055804b003full,
    0x400055004b0040ull, 0x410055004b0041ull, 0x5400540054004bull, 0x530012000a004dull, 0x4b0055004d004bull, 0x5300130009004dull, 0x4b0055004d004bull, 0x53004b0038004bull,
    0x5400540054004cull, 0x5300330012004dull, 0x4c0055004d004cull, 0x5300320013004dull, 0x4c0055004d004cull, 0x4b004c001e004bull, 0x400055804b0040ull, 0x3f0055804b003full,
    0x41004b00590041ull, 0x40003f80030040ull, 0x41003f80060041ull, 0x41004080070041ull, 0x53000800410041ull, 0x40004180050040ull, 0x53000400400040ull, 0x3f00408001003full,
    0x3f00418002003full, 0x530000003f003full, 0x32005500390032ull, 0x32003c005a0032ull, 0x32003f005b0032ull, 0x330055003a0033ull, 0x33003d005a0033ull, 0x330040005b0033ull,
    0x340055003b0034ull, 0x34003e005a0034ull, 0x340041005b0034ull,
};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "chapman_shipped";
  static constexpr int NS = 4;      // species including fixed ones
  static constexpr int NV = 3;      // variable species (solved system)
  static constexpr int NR = 4;      // reactions
  static constexpr int NP = 2;      // runtime parameter slots per cell
  static constexpr int NPH = 2;      // photolysis slots
  static constexpr int NFIX = 1;
  static constexpr int NLU = 9;
  static constexpr int NSTAGE = 3;
  static constexpr bool RUNTIME_ENV = false;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.435866521508459;
  static constexpr double ELO = 3.0;
  static constexpr double SEED = 9.9999999999999995e-07;
  static constexpr double ENV_T = 298.14999999999998;
  static constexpr double ENV_RHO = 2.46e+19;
  static constexpr long long LU_FMA = 5;
  static constexpr long long LU_SCALE = 3;
  static constexpr long long SOLVE_L = 3;
  static constexpr long long SOLVE_U = 3;
  static constexpr long long FUN_FLOPS = 28;
  static constexpr long long JAC_FLOPS = 38;

  __host__ __device__ static constexpr int var_phys(int i) { constexpr int t[3] = {2, 0, 1}; return t[i]; }
  __host__ __device__ static constexpr int fix_phys(int i) { constexpr int t[1] = {3}; return t[i]; }
  __host__ __device__ static constexpr double atol_v(int i) { constexpr double t[3] = {0.001, 0.001, 0.001}; return t[i]; }
  __host__ __device__ static constexpr double rtol_v(int i) { constexpr double t[3] = {9.9999999999999995e-07, 9.9999999999999995e-07, 9.9999999999999995e-07}; return t[i]; }
  static constexpr double ATOL[NS] = {0.001, 0.001, 0.001, 0.001};
  static constexpr double RTOL[NS] = {9.9999999999999995e-07, 9.9999999999999995e-07, 9.9999999999999995e-07, 9.9999999999999995e-07};
  __host__ __device__ static constexpr int lu_prow(int s) { constexpr int t[9] = {2, 2, 2, 0, 0, 0, 1, 1, 1}; return t[s]; }
  __host__ __device__ static constexpr int lu_pcol(int s) { constexpr int t[9] = {2, 0, 1, 2, 0, 1, 2, 0, 1}; return t[s]; }
  static const char* species_name(int s) { static const char* t[4] = {"O", "O2", "O3", "M"}; return t[s]; }
  static const char* photolysis_name(int p) { static const char* t[2] = {"J_1", "J_2"}; return t[p]; }

  // Rate constants of every reaction (reaction index order).  P(n) is the
  // cell's runtime parameter n (photolysis J_n or external Rate slot n),
  // FIX(s) the concentration of fixed species s, T/RHO the cell's
  // temperature and air density.
  template <class PA, class FA, class KO>
  __device__ __forceinline__ static void rate_constants(const PA& P, const FA& FIX, double T, double RHO,
                                                      double RH, double CLW, KO& k) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX;
    k.set(0, P(0));
    k.set(1, 6.0e-34*FIX(3));
    k.set(2, P(1));
    k.set(3, 7.9999999999999998e-12);
  }

  // Per-cell working storage, in slots of one double: the LU factors, the
  // state y, the stage vectors K_1..K_s, the tendency F, the increment dy and
  // the rate constants of the current host step.
  static constexpr int Y = 9;
  static constexpr int K0 = 12;
  static constexpr int F = 21;
  static constexpr int DY = 24;
  static constexpr int KT = 27;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 31;
  static constexpr bool TABLE_ATTEMPT = false;

  // Mass-action tendencies F(y) of the variable species (logical order):
  // y(i) supplies the state, out(i, F_i) receives the result.
  template <class YA, class KA, class FO>
  __device__ __forceinline__ static void fun(const YA& y, const KA& k, FO&& out) {
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double q0 = k(0) * y2;
    const double q1 = k(1) * y1 * y2;
    const double q2 = k(2) * y0;
    const double q3 = k(3) * y1 * y0;
    out(0, q1 - q2 - q3);
    out(1, 2.0 * q0 - q1 + q2 - q3);
    out(2, fma(2.0, q3, -q0 - q1 + q2));
  }

  // W = I/(gamma h) - J(y) into the LU slots that hold W entries.
  template <class YA, class KA, class SA>
  __device__ __forceinline__ static void jac_w(const YA& y, const KA& k, double inv_g_dt, SA& S) {
    (void)inv_g_dt;
    const double y0 = y(0);
    const double y1 = y(1);
    const double y2 = y(2);
    const double d0_2 = k(0);
    const double d1_1 = k(1) * y2;
    const double d1_2 = k(1) * y1;
    const double d2_0 = k(2);
    const double d3_1 = k(3) * y0;
    const double d3_0 = k(3) * y1;
    S[0] = inv_g_dt + d2_0 + d3_0;
    S[1] = -d1_1 + d3_1;
    S[2] = -d1_2;
    S[3] = -d2_0 + d3_0;
    S[4] = inv_g_dt + d1_1 + d3_1;
    S[5] = -2.0 * d0_2 + d1_2;
    S[6] = fma(-2.0, d3_0, -d2_0);
    S[7] = fma(-2.0, d3_1, d1_1);
    S[8] = inv_g_dt + d0_2 + d1_2;
  }

  // Physical (row, column) of every W slot, for the dense Jacobian.
  template <class Fn>
  __device__ __forceinline__ static void for_each_w_slot(Fn&& fn) {
    fn(0, 2, 2);
    fn(1, 2, 0);
    fn(2, 2, 1);
    fn(3, 0, 2);
    fn(4, 0, 0);
    fn(5, 0, 1);
    fn(6, 1, 2);
    fn(7, 1, 0);
    fn(8, 1, 1);
  }

  // Fixed-species columns of the dense Jacobian: dF_i/dC_f through the
  // rate constants' dependence on fixed species (third bodies).
  template <class PA, class FA, class YA, class Fn>
  __device__ __forceinline__ static void jac_fixed_columns(const PA& P, const FA& FIX, double T, double RHO,
                                                         double RH, double CLW, const YA& y, Fn&& fn) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX; (void)y;
    fn(0, 3, -((6.0e-34) * y(1) * y(2)));
    fn(1, 3, -((6.0e-34) * y(1) * y(2)));
    fn(2, 3, ((6.0e-34) * y(1) * y(2)));
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
      double v3 = S[3];
      double v6 = S[6];
      S[3] = v3 * rd;
      S[6] = v6 * rd;
    }
    {  // pivot row 1
      const double a3 = S[3];
      const double u4 = fma(-a3, S[1], S[4]);
      ok = ok && (u4 != 0.0);
      const double rd = 1.0 / u4;
      S[4] = rd;
      double v5 = S[5];
      v5 = fma(-a3, S[2], v5);
      S[5] = v5;
      const double b1 = S[1];
      double v7 = S[7];
      v7 = fma(-S[6], b1, v7);
      S[7] = v7 * rd;
    }
    {  // pivot row 2
      const double a6 = S[6];
      const double a7 = S[7];
      const double u8 = fma(-a7, S[5], fma(-a6, S[2], S[8]));
      ok = ok && (u8 != 0.0);
      const double rd = 1.0 / u8;
      S[8] = rd;
    }
    return ok;
  }

  // Solve (LU) x = b in place on slots [base, base + NV): unit-L forward
  // sweep, then the U backward sweep scaled by the stored 1/U_ii.
  template <class SA>
  __device__ __forceinline__ static void solve(SA& S, const int base) {
    const double v0 = S[base + 0];
    const double v1 = fma(-S[3], v0, S[base + 1]);
    const double v2 = fma(-S[7], v1, fma(-S[6], v0, S[base + 2]));
    const double x2 = (v2) * S[8];
    S[base + 2] = x2;
    const double x1 = (fma(-S[5], x2, v1)) * S[4];
    S[base + 1] = x1;
    const double x0 = (fma(-S[2], x2, fma(-S[1], x1, v0))) * S[0];
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
      S[12 + i] = S[F + i];
    }
    solve(S, 12);
    fun([&](int i) { return S[Y + i] + S[12 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c21 = -1.0156171083877703 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[15 + i] = fma(c21, S[12 + i], S[F + i]);
    }
    solve(S, 15);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[18 + i] = fma(c32, S[15 + i], fma(c31, S[12 + i], S[F + i]));
    }
    solve(S, 18);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[12 + i];
      const double k1 = S[15 + i];
      const double k2 = S[18 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
      err_sq = fma(q, q, err_sq);
    }
    return fmax(sqrt(err_sq / 4.0), 1.0e-10);
  }

  // Step-size factor from the error norm (integrate.j2:324-333).
  __device__ __forceinline__ static double growth(double err) {
    const double fac = 0.9 / cbrt(err);
    return fmax(0.2, fmin(fac, 6.0));
  }

  // ---- warp-cooperative attempt (static warp schedules) ----
  static constexpr int NPART = 6;
  static constexpr int Q = 31;            // rates q_r, then q_i of the error norm
  static constexpr int D = 35;     // partial derivatives
  static constexpr int CB = 41;        // constants
  static constexpr int NCONST = 9;
  static constexpr int COOP_SLOTS = CB + NCONST;
  // Run steps [s_begin, s_end) of the static warp schedule on S: one
  // uniform operation S[out] = fma(+-S[a], S[b], S[c]) (or a pivot
  // reciprocal) per lane and step, a warp barrier between steps.  The words
  // of the next SCHED_AHEAD steps are in flight while the current ones
  // execute; words past the end read as idle lanes.  Returns false if a
  // reciprocal met a zero pivot.
  static constexpr int SCHED_AHEAD = 8;
  __device__ __forceinline__ static bool run_schedule(double* S, int s_begin, int s_end, unsigned lane) {
    const unsigned long long* __restrict__ T = coop::sched;
    bool ok = true;
    unsigned long long cur[SCHED_AHEAD];
    #pragma unroll
    for (int j = 0; j < SCHED_AHEAD; ++j) {
      const int s = s_begin + j;
      cur[j] = s < s_end ? __ldg(T + (size_t)s * 32 + lane) : 0xffffull;
    }
    for (int s0 = s_begin; s0 < s_end; s0 += SCHED_AHEAD) {
      unsigned long long nxt[SCHED_AHEAD];
      #pragma unroll
      for (int j = 0; j < SCHED_AHEAD; ++j) {
        const int s = s0 + SCHED_AHEAD + j;
        nxt[j] = s < s_end ? __ldg(T + (size_t)s * 32 + lane) : 0xffffull;
      }
      #pragma unroll
      for (int j = 0; j < SCHED_AHEAD; ++j) {
        const unsigned long long w = cur[j];
        const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
        const unsigned out = lo & 0xffffu;
        if (out != 0xffffu) {
          if (hi >> 31) {
            const double v = S[out];
            ok = ok && (v != 0.0);
            S[out] = 1.0 / v;
          } else {
            // Negation flips the sign bit: exact, like -x in the per-thread code.
            const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                                  ((long long)(lo >> 31) << 63));
            S[out] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
          }
        }
        __syncwarp();
      }
      #pragma unroll
      for (int j = 0; j < SCHED_AHEAD; ++j) cur[j] = nxt[j];
    }
    return ok;
  }

  // One attempt by a whole warp on the cell held in shared memory S
  // (COOP_SLOTS doubles; the rate constants in the KT slots).  Same values
  // as attempt(); the error norm is summed by lane 0 in species order.
  // Returns err on every lane.
  template <class KA>
  __device__ __forceinline__ static double attempt_coop(double* S, const KA& k, double h, int& status,
                                                       unsigned lane) {
    (void)k;
    namespace T = coop;
    for (int i = lane; i < NCONST; i += 32) S[CB + i] = T::const_val[i];
    __syncwarp();
    if (lane == 0) {
      S[CB + 3] = 1.0 / (GAMMA * h);
      S[45] = -1.0156171083877703 / h;    // c21 / h
      S[46] = 4.0759956452537702 / h;    // c31 / h
      S[47] = 9.20767942983308 / h;    // c32 / h
    }
    __syncwarp();
    bool ok = true;
    for (int st = 0; st < NSTAGE; ++st) ok = run_schedule(S, T::stage_step[st], T::stage_step[st + 1], lane) && ok;
    if (__any_sync(0xffffffffu, !ok)) status |= 1;
    // Increment, and q_i^2 of the error norm into the rate slots.
    for (int i = lane; i < NV; i += 32) {
      const double k0 = S[12 + i];
      const double k1 = S[15 + i];
      const double k2 = S[18 + i];
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
      err = fmax(sqrt(err_sq / 4.0), 1.0e-10);
    }
    return __shfl_sync(0xffffffffu, err, 0);
  }

  // ---- tangent of one accepted step (forward sensitivities) ----
  static constexpr int DYT = 50;     // dy in, dy_new out (NV)
  static constexpr int DKR = 53;     // dk, the rate constants' tangent (NR)
  static constexpr int TLM_CB = 83;  // constants of the tangent program
  static constexpr int TLM_NCONST = 9;
  static constexpr int NSLOTS_TLM = 92;
  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks
  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and
  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].
  template <class SA, class KA>
  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {
    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);
    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];
    S[86] = -1.0156171083877703 / h;    // c21 / h
    S[87] = 4.0759956452537702 / h;    // c31 / h
    S[88] = 9.20767942983308 / h;    // c32 / h
    for (int n = 0; n < coop::TLM_OPS; ++n) {
      const unsigned long long w = __ldg(coop::tlm_prog + n);
      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                            ((long long)(lo >> 31) << 63));
      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
    }
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 31;      // dL/dy
  static constexpr int KBAR = 34;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 43;    // adjoint of the pending stage tendency
  static constexpr int KB = 46;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 50;
  // Solve W^T x = b in place on [base, base + NV) with the stored LU of W.
  template <class SA>
  __device__ __forceinline__ static void solve_t(SA& S, const int base) {
    const double z0 = (S[base + 0]) * S[0];
    const double z1 = (fma(-S[1], z0, S[base + 1])) * S[4];
    const double z2 = (fma(-S[5], z1, fma(-S[2], z0, S[base + 2]))) * S[8];
    const double x2 = z2;
    S[base + 2] = x2;
    const double x1 = fma(-S[7], x2, z1);
    S[base + 1] = x1;
    const double x0 = fma(-S[6], x2, fma(-S[3], x1, z0));
    S[base + 0] = x0;
  }

  // u^T J(y) v terms of stage i: y in S[Y..], u in S[ub..], v = K_i in S[vb..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adj_wterm(SA& S, const KA& k, const int ub, const int vb) {
    auto u = [&](int i) { return S[ub + i]; };
    const double y0 = S[Y + 0];
    const double v0 = S[vb + 0];
    const double y1 = S[Y + 1];
    const double v1 = S[vb + 1];
    const double y2 = S[Y + 2];
    const double v2 = S[vb + 2];
    { const double s = fma(2.0, u(1), -u(2));
      S[KB + 0] = fma(s, v2, S[KB + 0]);
      const double ks = k(0) * s;
    }
    { const double s = -u(1) - u(2) + u(0);
      S[KB + 1] = fma(s, (y2) * v1 + (y1) * v2, S[KB + 1]);
      const double ks = k(1) * s;
      S[LAM + 1] = fma(ks, v2, S[LAM + 1]);
      S[LAM + 2] = fma(ks, v1, S[LAM + 2]);
    }
    { const double s = -u(0) + u(1) + u(2);
      S[KB + 2] = fma(s, v0, S[KB + 2]);
      const double ks = k(2) * s;
    }
    { const double s = fma(2.0, u(2), -u(1) - u(0));
      S[KB + 3] = fma(s, (y1) * v0 + (y0) * v1, S[KB + 3]);
      const double ks = k(3) * s;
      S[LAM + 0] = fma(ks, v1, S[LAM + 0]);
      S[LAM + 1] = fma(ks, v0, S[LAM + 1]);
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
    const double s0 = fma(2.0, fb(1), -fb(2));
    S[KB + 0] = fma(s0, y2, S[KB + 0]);
    const double s1 = -fb(1) - fb(2) + fb(0);
    S[KB + 1] = fma(s1, y1 * y2, S[KB + 1]);
    const double s2 = -fb(0) + fb(1) + fb(2);
    S[KB + 2] = fma(s2, y0, S[KB + 2]);
    const double s3 = fma(2.0, fb(2), -fb(1) - fb(0));
    S[KB + 3] = fma(s3, y0 * y1, S[KB + 3]);
    ybar(0, k(2) * s2 + k(3) * s3 * y1);
    ybar(1, k(1) * s1 * y2 + k(3) * s3 * y0);
    ybar(2, k(0) * s0 + k(1) * s1 * y1);
  }

  // Reverse of one accepted step of size h.  Requires the values attempt()
  // left in S for this step (LU, K_i) and y_n in S[Y..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 3 + j] = 6.1697947043828245 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 6 + j] = -0.42772256543218573 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 6);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 6, 18);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 6 + j];
    { const double cc = 4.0759956452537702 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 0 + q]); }
    { const double cc = 9.20767942983308 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 3 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 3 + q]); }
    // stage 2
    solve_t(S, KBAR + 3);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 3, 15);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 3 + j];
    { const double cc = -1.0156171083877703 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 3 + q], S[KBAR + 0 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + S[12 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(1.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 1
    solve_t(S, KBAR + 0);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 0, 12);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 0 + j];
    adj_fterm(S, k, [&](int q) { return S[Y + q]; },
              [&](int j, double x) { S[LAM + j] += x; });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
  }
};

}  // namespace mkpp_chapman_shipped
