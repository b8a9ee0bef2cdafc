// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/chapman_rodas3.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 4 species (3 variable), 4 reactions, 9 W slots, 9 LU slots, 5 LU products, 3 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_chapman_rodas3 {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const double const_val[12] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -2.0, 2.0};
static __device__ const int stage_step[5] = {0, 16, 26, 44, 64};
static __device__ const unsigned long long sched[2048] = {
    0x2c002e001e0026ull, 0x2c000b001f0027ull, 0x2c000a001f0028ull, 0x2c002e00200029ull, 0x2c00090021002aull, 0x2c000a0021002bull, 0x2c000b001e0022ull, 0x2c000a001f0023ull,
    0x2c000900200024ull, 0x2c000a00210025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2f002e00290000ull, 0x2c002e80270001ull, 0x2c002e80280002ull, 0x2c002e80290003ull, 0x2f002e00270004ull, 0x2c003600260005ull, 0x2c002e80290006ull, 0x2c002e00270007ull,
    0x2f002e00260008ull, 0x2c000b00230023ull, 0x2c000900250025ull, 0x2c003700220019ull, 0x2c002e8022001aull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2e002b0000ull, 0x1002e002a0001ull, 0x3002e002b0003ull, 0x4002e002a0004ull, 0x5002e00280005ull, 0x6002b00360006ull, 0x7002a00360007ull, 0x8002e00280008ull,
    0x2c002e00230018ull, 0x19002e80230019ull, 0x1a002e8023001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000000ull, 0x18002e80240018ull, 0x19002e00240019ull, 0x1a002e0024001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000000030003ull, 0x2c000000060006ull, 0x18002e80250018ull, 0x19002e80250019ull, 0x1a00250037001aull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4000180030004ull, 0x5000280030005ull, 0x7000180060007ull, 0x8000280060008ull, 0x2c002e0018000cull, 0x2c002e0019000dull, 0x2c002e001a000eull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000004ull, 0xd000c8003000dull, 0xe000c8006000eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000400070007ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c0008000e000eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xd000e8005000dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c0004000d000dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c0000000c000cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e0018000full, 0x2c002e00190010ull, 0x2c002e001a0011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xf000c0030000full, 0x10000d00300010ull, 0x11000e00300011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c000800110011ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x10001180050010ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000400100010ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c0000000f000full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c0037000c0022ull, 0x2c0037000d0023ull, 0x2c0037000e0024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x9002e0022001bull, 0xa002e0023001cull, 0xb002e0024001dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c001d001e0022ull, 0x2c001c001f0023ull, 0x2c001b00200024ull, 0x2c001c00210025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c001d00230023ull, 0x2c001b00250025ull, 0x2c003700220019ull, 0x2c002e8022001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e00230018ull, 0x19002e80230019ull, 0x1a002e8023001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x18002e80240018ull, 0x19002e00240019ull, 0x1a002e0024001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x18002e80250018ull, 0x19002e80250019ull, 0x1a00250037001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e00180012ull, 0x2c002e00190013ull, 0x2c002e001a0014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12000c00310012ull, 0x13000d00310013ull, 0x14000e00310014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x12000f00320012ull, 0x13001000320013ull, 0x14001100320014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c000800140014ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x13001480050013ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000400130013ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x2c000000120012ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c0037000c0022ull, 0x2c0037000d0023ull, 0x2c0037000e0024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x9002e0022001bull, 0xa002e0023001cull, 0xb002e0024001dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x1b002e0012001bull, 0x1c002e0013001cull, 0x1d002e0014001dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c001d001e0022ull, 0x2c001c001f0023ull, 0x2c001b00200024ull, 0x2c001c00210025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c001d00230023ull, 0x2c001b00250025ull, 0x2c003700220019ull, 0x2c002e8022001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e00230018ull, 0x19002e80230019ull, 0x1a002e8023001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x18002e80240018ull, 0x19002e00240019ull, 0x1a002e0024001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x18002e80250018ull, 0x19002e80250019ull, 0x1a00250037001aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e00180015ull, 0x2c002e00190016ull, 0x2c002e001a0017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15000c00330015ull, 0x16000d00330016ull, 0x17000e00330017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15000f00340015ull, 0x16001000340016ull, 0x17001100340017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15001200350015ull, 0x16001300350016ull, 0x17001400350017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x16001580030016ull, 0x17001580060017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x17001680070017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000800170017ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x16001780050016ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000400160016ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15001680010015ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x15001780020015ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c000000150015ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
};
constexpr int TLM_OPS = 419;
static __device__ const double tlm_const_val[10] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2.0};
static __device__ const unsigned long long tlm_prog[419] = {
    0x5d005d005d004bull, 0x5d005d005d004cull, 0x5d005d005d004dull, 0x5d005d005d0054ull, 0x5c005e003a0056ull, 0x54005e00560054ull, 0x5c0054001e0054ull, 0x5c005e000b0055ull,
    0x540055003b0054ull, 0x4d005e8054004dull, 0x4c00540065004cull, 0x5d005d005d0054ull, 0x5c0039000b0056ull, 0x54005e00560054ull, 0x5c003a000a0056ull, 0x54005e00560054ull,
    0x5c0054001f0054ull, 0x5c000b000a0055ull, 0x540055003c0054ull, 0x4c005e8054004cull, 0x4d005e8054004dull, 0x4b005e0054004bull, 0x5d005d005d0054ull, 0x5c005e00380056ull,
    0x54005e00560054ull, 0x5c005400200054ull, 0x5c005e00090055ull, 0x540055003d0054ull, 0x4b005e8054004bull, 0x4c005e0054004cull, 0x4d005e0054004dull, 0x5d005d005d0054ull,
    0x5c0038000a0056ull, 0x54005e00560054ull, 0x5c003900090056ull, 0x54005e00560054ull, 0x5c005400210054ull, 0x5c000a00090055ull, 0x540055003e0054ull, 0x4c005e8054004cull,
    0x4b005e8054004bull, 0x4d00540065004dull, 0x5c005e004b003full, 0x5c005e004c0040ull, 0x5c005e004d0041ull, 0x5d005d005d0054ull, 0x5c005e000e0056ull, 0x54005e00560054ull,
    0x5c0054003b0054ull, 0x5d005d005d0055ull, 0x540055001e0054ull, 0x41005e80540041ull, 0x40005400650040ull, 0x5d005d005d0054ull, 0x5c000d000b0056ull, 0x54005e00560054ull,
    0x5c000e000a0056ull, 0x54005e00560054ull, 0x5c0054003c0054ull, 0x5d005d005d0055ull, 0x5c003a000d0056ull, 0x55005e00560055ull, 0x5c0039000e0056ull, 0x55005e00560055ull,
    0x540055001f0054ull, 0x40005e80540040ull, 0x41005e80540041ull, 0x3f005e0054003full, 0x5d005d005d0054ull, 0x5c005e000c0056ull, 0x54005e00560054ull, 0x5c0054003d0054ull,
    0x5d005d005d0055ull, 0x54005500200054ull, 0x3f005e8054003full, 0x40005e00540040ull, 0x41005e00540041ull, 0x5d005d005d0054ull, 0x5c000c000a0056ull, 0x54005e00560054ull,
    0x5c000d00090056ull, 0x54005e00560054ull, 0x5c0054003e0054ull, 0x5d005d005d0055ull, 0x5c0039000c0056ull, 0x55005e00560055ull, 0x5c0038000d0056ull, 0x55005e00560055ull,
    0x54005500210054ull, 0x40005e80540040ull, 0x3f005e8054003full, 0x41005400650041ull, 0x40003f80030040ull, 0x41003f80060041ull, 0x41004080070041ull, 0x5c000800410041ull,
    0x40004180050040ull, 0x5c000400400040ull, 0x3f00408001003full, 0x3f00418002003full, 0x5c0000003f003full, 0x5c005e004b0042ull, 0x42003f005f0042ull, 0x5c005e004c0043ull,
    0x430040005f0043ull, 0x5c005e004d0044ull, 0x440041005f0044ull, 0x5d005d005d0054ull, 0x5c005e00110056ull, 0x54005e00560054ull, 0x5c0054003b0054ull, 0x5d005d005d0055ull,
    0x540055001e0054ull, 0x44005e80540044ull, 0x43005400650043ull, 0x5d005d005d0054ull, 0x5c0010000b0056ull, 0x54005e00560054ull, 0x5c0011000a0056ull, 0x54005e00560054ull,
    0x5c0054003c0054ull, 0x5d005d005d0055ull, 0x5c003a00100056ull, 0x55005e00560055ull, 0x5c003900110056ull, 0x55005e00560055ull, 0x540055001f0054ull, 0x43005e80540043ull,
    0x44005e80540044ull, 0x42005e00540042ull, 0x5d005d005d0054ull, 0x5c005e000f0056ull, 0x54005e00560054ull, 0x5c0054003d0054ull, 0x5d005d005d0055ull, 0x54005500200054ull,
    0x42005e80540042ull, 0x43005e00540043ull, 0x44005e00540044ull, 0x5d005d005d0054ull, 0x5c000f000a0056ull, 0x54005e00560054ull, 0x5c001000090056ull, 0x54005e00560054ull,
    0x5c0054003e0054ull, 0x5d005d005d0055ull, 0x5c0039000f0056ull, 0x55005e00560055ull, 0x5c003800100056ull, 0x55005e00560055ull, 0x54005500210054ull, 0x43005e80540043ull,
    0x42005e80540042ull, 0x44005400650044ull, 0x43004280030043ull, 0x44004280060044ull, 0x44004380070044ull, 0x5c000800440044ull, 0x43004480050043ull, 0x5c000400430043ull,
    0x42004380010042ull, 0x42004480020042ull, 0x5c000000420042ull, 0x5c005e0009004eull, 0x5c005e00380051ull, 0x4e000c0065004eull, 0x51003f00650051ull, 0x5c005e000a004full,
    0x5c005e00390052ull, 0x4f000d0065004full, 0x52004000650052ull, 0x5c005e000b0050ull, 0x5c005e003a0053ull, 0x50000e00650050ull, 0x53004100650053ull, 0x5d005d005d004bull,
    0x5d005d005d004cull, 0x5d005d005d004dull, 0x5d005d005d0054ull, 0x5c005e00530056ull, 0x54005e00560054ull, 0x5c0054001e0054ull, 0x5c005e00500055ull, 0x540055003b0054ull,
    0x4d005e8054004dull, 0x4c00540065004cull, 0x5d005d005d0054ull, 0x5c005200500056ull, 0x54005e00560054ull, 0x5c0053004f0056ull, 0x54005e00560054ull, 0x5c0054001f0054ull,
    0x5c0050004f0055ull, 0x540055003c0054ull, 0x4c005e8054004cull, 0x4d005e8054004dull, 0x4b005e0054004bull, 0x5d005d005d0054ull, 0x5c005e00510056ull, 0x54005e00560054ull,
    0x5c005400200054ull, 0x5c005e004e0055ull, 0x540055003d0054ull, 0x4b005e8054004bull, 0x4c005e0054004cull, 0x4d005e0054004dull, 0x5d005d005d0054ull, 0x5c0051004f0056ull,
    0x54005e00560054ull, 0x5c0052004e0056ull, 0x54005e00560054ull, 0x5c005400210054ull, 0x5c004f004e0055ull, 0x540055003e0054ull, 0x4c005e8054004cull, 0x4b005e8054004bull,
    0x4d00540065004dull, 0x5c005e004b0045ull, 0x45003f00600045ull, 0x45004200610045ull, 0x5c005e004c0046ull, 0x46004000600046ull, 0x46004300610046ull, 0x5c005e004d0047ull,
    0x47004100600047ull, 0x47004400610047ull, 0x5d005d005d0054ull, 0x5c005e00140056ull, 0x54005e00560054ull, 0x5c0054003b0054ull, 0x5d005d005d0055ull, 0x540055001e0054ull,
    0x47005e80540047ull, 0x46005400650046ull, 0x5d005d005d0054ull, 0x5c0013000b0056ull, 0x54005e00560054ull, 0x5c0014000a0056ull, 0x54005e00560054ull, 0x5c0054003c0054ull,
    0x5d005d005d0055ull, 0x5c003a00130056ull, 0x55005e00560055ull, 0x5c003900140056ull, 0x55005e00560055ull, 0x540055001f0054ull, 0x46005e80540046ull, 0x47005e80540047ull,
    0x45005e00540045ull, 0x5d005d005d0054ull, 0x5c005e00120056ull, 0x54005e00560054ull, 0x5c0054003d0054ull, 0x5d005d005d0055ull, 0x54005500200054ull, 0x45005e80540045ull,
    0x46005e00540046ull, 0x47005e00540047ull, 0x5d005d005d0054ull, 0x5c0012000a0056ull, 0x54005e00560054ull, 0x5c001300090056ull, 0x54005e00560054ull, 0x5c0054003e0054ull,
    0x5d005d005d0055ull, 0x5c003900120056ull, 0x55005e00560055ull, 0x5c003800130056ull, 0x55005e00560055ull, 0x54005500210054ull, 0x46005e80540046ull, 0x45005e80540045ull,
    0x47005400650047ull, 0x46004580030046ull, 0x47004580060047ull, 0x47004680070047ull, 0x5c000800470047ull, 0x46004780050046ull, 0x5c000400460046ull, 0x45004680010045ull,
    0x45004780020045ull, 0x5c000000450045ull, 0x5c005e0009004eull, 0x5c005e00380051ull, 0x4e000c0065004eull, 0x51003f00650051ull, 0x4e005e0012004eull, 0x51005e00450051ull,
    0x5c005e000a004full, 0x5c005e00390052ull, 0x4f000d0065004full, 0x52004000650052ull, 0x4f005e0013004full, 0x52005e00460052ull, 0x5c005e000b0050ull, 0x5c005e003a0053ull,
    0x50000e00650050ull, 0x53004100650053ull, 0x50005e00140050ull, 0x53005e00470053ull, 0x5d005d005d004bull, 0x5d005d005d004cull, 0x5d005d005d004dull, 0x5d005d005d0054ull,
    0x5c005e00530056ull, 0x54005e00560054ull, 0x5c0054001e0054ull, 0x5c005e00500055ull, 0x540055003b0054ull, 0x4d005e8054004dull, 0x4c00540065004cull, 0x5d005d005d0054ull,
    0x5c005200500056ull, 0x54005e00560054ull, 0x5c0053004f0056ull, 0x54005e00560054ull, 0x5c0054001f0054ull, 0x5c0050004f0055ull, 0x540055003c0054ull, 0x4c005e8054004cull,
    0x4d005e8054004dull, 0x4b005e0054004bull, 0x5d005d005d0054ull, 0x5c005e00510056ull, 0x54005e00560054ull, 0x5c005400200054ull, 0x5c005e004e0055ull, 0x540055003d0054ull,
    0x4b005e8054004bull, 0x4c005e0054004cull, 0x4d005e0054004dull, 0x5d005d005d0054ull, 0x5c0051004f0056ull, 0x54005e00560054ull, 0x5c0052004e0056ull, 0x54005e00560054ull,
    0x5c005400210054ull, 0x5c004f004e0055ull, 0x540055003e0054ull, 0x4c005e8054004cull, 0x4b005e8054004bull, 0x4d00540065004dull, 0x5c005e004b0048ull, 0x48003f00620048ull,
    0x48004200630048ull, 0x48004500640048ull, 0x5c005e004c0049ull, 0x49004000620049ull, 0x49004300630049ull, 0x49004600640049ull, 0x5c005e004d004aull, 0x4a00410062004aull,
    0x4a00440063004aull, 0x4a00470064004aull, 0x5d005d005d0054ull, 0x5c005e00170056ull, 0x54005e00560054ull, 0x5c0054003b0054ull, 0x5d005d005d0055ull, 0x540055001e0054ull,
    0x4a005e8054004aull, 0x49005400650049ull, 0x5d005d005d0054ull, 0x5c0016000b0056ull, 0x54005e00560054ull, 0x5c0017000a0056ull, 0x54005e00560054ull, 0x5c0054003c0054ull,
    0x5d005d005d0055ull, 0x5c003a00160056ull, 0x55005e00560055ull, 0x5c003900170056ull, 0x55005e00560055ull, 0x540055001f0054ull, 0x49005e80540049ull, 0x4a005e8054004aull,
    0x48005e00540048ull, 0x5d005d005d0054ull, 0x5c005e00150056ull, 0x54005e00560054ull, 0x5c0054003d0054ull, 0x5d005d005d0055ull, 0x54005500200054ull, 0x48005e80540048ull,
    0x49005e00540049ull, 0x4a005e0054004aull, 0x5d005d005d0054ull, 0x5c0015000a0056ull, 0x54005e00560054ull, 0x5c001600090056ull, 0x54005e00560054ull, 0x5c0054003e0054ull,
    0x5d005d005d0055ull, 0x5c003900150056ull, 0x55005e00560055ull, 0x5c003800160056ull, 0x55005e00560055ull, 0x54005500210054ull, 0x49005e80540049ull, 0x48005e80540048ull,
    0x4a00540065004aull, 0x49004880030049ull, 0x4a00488006004aull, 0x4a00498007004aull, 0x5c0008004a004aull, 0x49004a80050049ull, 0x5c000400490049ull, 0x48004980010048ull,
    0x48004a80020048ull, 0x5c000000480048ull, 0x38003f00650038ull, 0x38005e00450038ull, 0x38005e00480038ull, 0x39004000650039ull, 0x39005e00460039ull, 0x39005e00490039ull,
    0x3a00410065003aull, 0x3a005e0047003aull, 0x3a005e004a003aull,
};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "chapman_rodas3";
  static constexpr int NS = 4;      // species including fixed ones
  static constexpr int NV = 3;      // variable species (solved system)
  static constexpr int NR = 4;      // reactions
  static constexpr int NP = 2;      // runtime parameter slots per cell
  static constexpr int NPH = 2;      // photolysis slots
  static constexpr int NFIX = 1;
  static constexpr int NLU = 9;
  static constexpr int NSTAGE = 4;
  static constexpr bool RUNTIME_ENV = false;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.5;
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
  __host__ __device__ static constexpr double atol_v(int i) { constexpr double t[3] = {1.0, 1.0, 1.0}; return t[i]; }
  __host__ __device__ static constexpr double rtol_v(int i) { constexpr double t[3] = {0.001, 0.001, 0.001}; return t[i]; }
  static constexpr double ATOL[NS] = {1.0, 1.0, 1.0, 1.0};
  static constexpr double RTOL[NS] = {0.001, 0.001, 0.001, 0.001};
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
  static constexpr int F = 24;
  static constexpr int DY = 27;
  static constexpr int KT = 30;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 34;
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
    const double c21 = 4.0 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[15 + i] = fma(c21, S[12 + i], S[F + i]);
    }
    solve(S, 15);
    fun([&](int i) { return S[Y + i] + 2.0 * S[12 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c31 = 1.0 / h;
    const double c32 = -1.0 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[18 + i] = fma(c32, S[15 + i], fma(c31, S[12 + i], S[F + i]));
    }
    solve(S, 18);
    fun([&](int i) { return S[Y + i] + 2.0 * S[12 + i] + S[18 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c41 = 1.0 / h;
    const double c42 = -1.0 / h;
    const double c43 = -2.6666666666666665 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[21 + i] = fma(c43, S[18 + i], fma(c42, S[15 + i], fma(c41, S[12 + i], S[F + i])));
    }
    solve(S, 21);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[12 + i];
      const double k1 = S[15 + i];
      const double k2 = S[18 + i];
      const double k3 = S[21 + i];
      const double yi = S[Y + i];
      const double ynew = fma(2.0, k0, yi) + k2 + k3;
      S[DY + i] = 2.0 * k0 + k2 + k3;
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (k3) / sc;
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
  static constexpr int Q = 34;            // rates q_r, then q_i of the error norm
  static constexpr int D = 38;     // partial derivatives
  static constexpr int CB = 44;        // constants
  static constexpr int NCONST = 12;
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
      S[48] = 4.0 / h;    // c21 / h
      S[49] = 1.0 / h;    // c31 / h
      S[50] = -1.0 / h;    // c32 / h
      S[51] = 1.0 / h;    // c41 / h
      S[52] = -1.0 / h;    // c42 / h
      S[53] = -2.6666666666666665 / h;    // c43 / h
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
      const double k3 = S[21 + i];
      const double yi = S[Y + i];
      const double ynew = fma(2.0, k0, yi) + k2 + k3;
      S[DY + i] = 2.0 * k0 + k2 + k3;
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      S[Q + i] = (k3) / sc;
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
  static constexpr int DYT = 56;     // dy in, dy_new out (NV)
  static constexpr int DKR = 59;     // dk, the rate constants' tangent (NR)
  static constexpr int TLM_CB = 92;  // constants of the tangent program
  static constexpr int TLM_NCONST = 10;
  static constexpr int NSLOTS_TLM = 102;
  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks
  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and
  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].
  template <class SA, class KA>
  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {
    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);
    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];
    S[95] = 4.0 / h;    // c21 / h
    S[96] = 1.0 / h;    // c31 / h
    S[97] = -1.0 / h;    // c32 / h
    S[98] = 1.0 / h;    // c41 / h
    S[99] = -1.0 / h;    // c42 / h
    S[100] = -2.6666666666666665 / h;    // c43 / h
    for (int n = 0; n < coop::TLM_OPS; ++n) {
      const unsigned long long w = __ldg(coop::tlm_prog + n);
      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                            ((long long)(lo >> 31) << 63));
      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
    }
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 34;      // dL/dy
  static constexpr int KBAR = 37;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 49;    // adjoint of the pending stage tendency
  static constexpr int KB = 52;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 56;
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
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 2.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 3 + j] = 0.0;
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 6 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 9 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 4
    solve_t(S, KBAR + 9);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 9, 21);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 9 + j];
    { const double cc = 1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 9 + q], S[KBAR + 0 + q]); }
    { const double cc = -1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 3 + q] = fma(cc, S[KBAR + 9 + q], S[KBAR + 3 + q]); }
    { const double cc = -2.6666666666666665 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 6 + q] = fma(cc, S[KBAR + 9 + q], S[KBAR + 6 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + 2.0 * S[12 + q] + S[18 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(2.0, x, S[KBAR + 0 + j]); S[KBAR + 6 + j] = fma(1.0, x, S[KBAR + 6 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 6);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 6, 18);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 6 + j];
    { const double cc = 1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 0 + q]); }
    { const double cc = -1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 3 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 3 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + 2.0 * S[12 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(2.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 2
    solve_t(S, KBAR + 3);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 3, 15);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 3 + j];
    { const double cc = 4.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 3 + q], S[KBAR + 0 + q]); }
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

}  // namespace mkpp_chapman_rodas3
