// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/small_strato_rodas3.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 7 species (6 variable), 10 reactions, 26 W slots, 29 LU slots, 29 LU products, 13 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_small_strato_rodas3 {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const double const_val[12] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -2.0, 2.0};
static __device__ const int stage_step[5] = {0, 31, 52, 85, 120};
static __device__ const unsigned long long sched[3840] = {
    0x6a006c0047005bull, 0x6a001f0048005cull, 0x6a001e0048005dull, 0x6a006c0049005eull, 0x6a0020004a005full, 0x6a001e004a0060ull, 0x6a006c004b0061ull, 0x6a006c004c0062ull,
    0x6a0020004d0063ull, 0x6a001d004d0064ull, 0x6a0020004e0065ull, 0x6a0021004e0066ull, 0x6a001e004f0067ull, 0x6a0022004f0068ull, 0x6a006c00500069ull, 0x6b006b006b0014ull,
    0x6b006b006b0019ull, 0x6b006b006b0012ull, 0x6a001f00470051ull, 0x6a001e00480052ull, 0x6a002000490053ull, 0x6a001e004a0054ull, 0x6a0020004b0055ull, 0x6a001d004c0056ull,
    0x6a001d004d0057ull, 0x6a0021004e0058ull, 0x6a0022004f0059ull, 0x6a00220050005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6d006c00620000ull, 0x6a006c80610001ull, 0x6a006c80620002ull, 0x6d006c005c0003ull, 0x6a0074005b0004ull, 0x6a006c805e0005ull, 0x6a006c00670006ull, 0x6a007400630007ull,
    0x6a006c005c0008ull, 0x6d006c005b0009ull, 0x6a006c805e000aull, 0x6a006c8065000bull, 0x6a006c0063000dull, 0x6a006c805c000eull, 0x6a006c805d000full, 0x6d006c005e0010ull,
    0x6a006c00650011ull, 0x6a006c80680013ull, 0x6a006c00660015ull, 0x6d006c00650016ull, 0x6a006c80670017ull, 0x6a006c00680018ull, 0x6a006c8066001aull, 0x6d006c0067001cull,
    0x6a001f00520052ull, 0x6a002000540054ull, 0x6a002000570057ull, 0x6a002000580058ull, 0x6a001e00590059ull, 0x6a006c0055003bull, 0x6a00750051003cull, 0x6a006c8051003dull,
    0x6c00630000ull, 0x1006c00640001ull, 0x3006c005f0003ull, 0x4006c005d0004ull, 0x5006c00600005ull, 0x6006c80690006ull, 0x8005f00740008ull, 0x9006c005d0009ull,
    0xa00600074000aull, 0x6a006c8067000cull, 0xe006c005f000eull, 0x10006c00600010ull, 0x17006c80690017ull, 0x6a006c8065001bull, 0x1c006c0069001cull, 0x3b006c8056003bull,
    0x3c006c8052003cull, 0x3d006c8052003dull, 0x6a006c0052003eull, 0x6a006c8058003full, 0x6a006c00580040ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3006c00680003ull, 0x8006c80680008ull, 0xa006c8061000aull, 0x10006c00610010ull, 0x8000000000000000ull, 0x3b006c8057003bull, 0x3c006c0053003cull, 0x3d006c0053003dull,
    0x3e006c8053003eull, 0x3f006c0059003full, 0x40006c80590040ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xa00640074000aull, 0x10006c00640010ull, 0x6a000000020002ull, 0x6a000000070007ull, 0x6a0000000d000dull, 0x8000000000000003ull, 0x3c006c8054003cull, 0x3d00540075003dull,
    0x3e006c8054003eull, 0x3f006c005a003full, 0x40006c805a0040ull, 0x6a006c003b0023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xa006c8066000aull, 0x10006c00660010ull, 0x5000180020005ull, 0x6a000300080008ull, 0x6a0003000e000eull, 0x6a000300130013ull, 0x6a000300180018ull, 0x3c006c0056003cull,
    0x3d006c0055003dull, 0x3e006c8055003eull, 0x6a006c003f0027ull, 0x6a006c00400028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x9000480080009ull, 0xa00018007000aull, 0xc00068008000cull, 0xf0004800e000full, 0x14000480130014ull, 0x19000480180019ull, 0x100001800d0010ull, 0x120006800e0012ull,
    0x15000580130015ull, 0x1a00058018001aull, 0x17000680130017ull, 0x1c00068018001cull, 0x3c006c8059003cull, 0x3d00570075003dull, 0x3e006c8057003eull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000009ull, 0xa00058008000aull, 0x100005800e0010ull, 0x3c006c005a003cull, 0x3d006c0058003dull, 0x3e006c8058003eull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0009000f000full, 0x6a000900140014ull, 0x6a000900190019ull, 0x3d006c0059003dull, 0x6a006c003c0024ull, 0x6a006c003e0026ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x10000a800f0010ull, 0x11000b800f0011ull, 0x12000c800f0012ull, 0x15000a80140015ull, 0x1a000a8019001aull, 0x16000b80140016ull, 0x17000c80140017ull, 0x1b000b8019001bull,
    0x1c000c8019001cull, 0x6a006c003d0025ull, 0x24002380020024ull, 0x260023800d0026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000010ull, 0x25002380070025ull, 0x260024800e0026ull, 0x27002480130027ull, 0x28002480180028ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001000150015ull, 0x6a0010001a001aull, 0x25002480080025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x16001180150016ull, 0x17001280150017ull, 0x1b0011801a001bull, 0x1c0012801a001cull, 0x260025800f0026ull, 0x27002580140027ull, 0x28002580190028ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000016ull, 0x27002680150027ull, 0x280026801a0028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0016001b001bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x1c0017801b001cull, 0x280027801b0028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x800000000000001cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001c00280028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x27002880170027ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001600270027ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x26002780110026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x26002880120026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001000260026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250026800a0025ull, 0x23002680010023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250027800b0025ull, 0x6a000000230023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250028800c0025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000900250025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x24002580040024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x24002680050024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x24002880060024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000300240024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a006c003b0029ull, 0x6a006c003c002aull, 0x6a006c003d002bull, 0x6a006c003e002cull, 0x6a006c003f002dull, 0x6a006c0040002eull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x290023006e0029ull, 0x2a0024006e002aull, 0x2b0025006e002bull, 0x2c0026006e002cull, 0x2d0027006e002dull, 0x2e0028006e002eull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2a00298002002aull, 0x2b00298007002bull, 0x2c0029800d002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002a8008002bull, 0x2c002a800e002cull, 0x2d002a8013002dull, 0x2e002a8018002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002b800f002cull, 0x2d002b8014002dull, 0x2e002b8019002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2d002c8015002dull, 0x2e002c801a002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2e002d801b002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001c002e002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2d002e8017002dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0016002d002dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002d8011002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2c002e8012002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0010002c002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002c800a002bull, 0x29002c80010029ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002d800b002bull, 0x6a000000290029ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002e800c002bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0009002b002bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2a002b8004002aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2a002c8005002aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2a002e8006002aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a0003002a002aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a007500230051ull, 0x6a007500240052ull, 0x6a007500250053ull, 0x6a007500260054ull, 0x6a007500270055ull, 0x6a007500280056ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x1d006c00510041ull, 0x1e006c00520042ull, 0x1f006c00530043ull, 0x20006c00540044ull, 0x21006c00550045ull, 0x22006c00560046ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a004300470051ull, 0x6a004200480052ull, 0x6a004400490053ull, 0x6a0042004a0054ull, 0x6a0044004b0055ull, 0x6a0041004c0056ull, 0x6a0041004d0057ull, 0x6a0045004e0058ull,
    0x6a0046004f0059ull, 0x6a00460050005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a004300520052ull, 0x6a004400540054ull, 0x6a004400570057ull, 0x6a004400580058ull, 0x6a004200590059ull, 0x6a006c0055003bull, 0x6a00750051003cull, 0x6a006c8051003dull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3b006c8056003bull, 0x3c006c8052003cull, 0x3d006c8052003dull, 0x6a006c0052003eull, 0x6a006c8058003full, 0x6a006c00580040ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3b006c8057003bull, 0x3c006c0053003cull, 0x3d006c0053003dull, 0x3e006c8053003eull, 0x3f006c0059003full, 0x40006c80590040ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c8054003cull, 0x3d00540075003dull, 0x3e006c8054003eull, 0x3f006c005a003full, 0x40006c805a0040ull, 0x6a006c003b002full, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c0056003cull, 0x3d006c0055003dull, 0x3e006c8055003eull, 0x2f0023006f002full, 0x6a006c003f0033ull, 0x6a006c00400034ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c8059003cull, 0x3d00570075003dull, 0x3e006c8057003eull, 0x2f00290070002full, 0x330027006f0033ull, 0x340028006f0034ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c005a003cull, 0x3d006c0058003dull, 0x3e006c8058003eull, 0x33002d00700033ull, 0x34002e00700034ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3d006c0059003dull, 0x6a006c003c0030ull, 0x6a006c003e0032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x300024006f0030ull, 0x6a006c003d0031ull, 0x320026006f0032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x30002a00700030ull, 0x310025006f0031ull, 0x32002c00700032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x31002b00700031ull, 0x30002f80020030ull, 0x32002f800d0032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x31002f80070031ull, 0x320030800e0032ull, 0x33003080130033ull, 0x34003080180034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x31003080080031ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x320031800f0032ull, 0x33003180140033ull, 0x34003180190034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x33003280150033ull, 0x340032801a0034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x340033801b0034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001c00340034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x33003480170033ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001600330033ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x32003380110032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x32003480120032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001000320032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310032800a0031ull, 0x2f00328001002full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310033800b0031ull, 0x6a0000002f002full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310034800c0031ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000900310031ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x30003180040030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x30003280050030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x30003480060030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000300300030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a007500230051ull, 0x6a007500240052ull, 0x6a007500250053ull, 0x6a007500260054ull, 0x6a007500270055ull, 0x6a007500280056ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x1d006c00510041ull, 0x1e006c00520042ull, 0x1f006c00530043ull, 0x20006c00540044ull, 0x21006c00550045ull, 0x22006c00560046ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x41006c002f0041ull, 0x42006c00300042ull, 0x43006c00310043ull, 0x44006c00320044ull, 0x45006c00330045ull, 0x46006c00340046ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a004300470051ull, 0x6a004200480052ull, 0x6a004400490053ull, 0x6a0042004a0054ull, 0x6a0044004b0055ull, 0x6a0041004c0056ull, 0x6a0041004d0057ull, 0x6a0045004e0058ull,
    0x6a0046004f0059ull, 0x6a00460050005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a004300520052ull, 0x6a004400540054ull, 0x6a004400570057ull, 0x6a004400580058ull, 0x6a004200590059ull, 0x6a006c0055003bull, 0x6a00750051003cull, 0x6a006c8051003dull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3b006c8056003bull, 0x3c006c8052003cull, 0x3d006c8052003dull, 0x6a006c0052003eull, 0x6a006c8058003full, 0x6a006c00580040ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3b006c8057003bull, 0x3c006c0053003cull, 0x3d006c0053003dull, 0x3e006c8053003eull, 0x3f006c0059003full, 0x40006c80590040ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c8054003cull, 0x3d00540075003dull, 0x3e006c8054003eull, 0x3f006c005a003full, 0x40006c805a0040ull, 0x6a006c003b0035ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c0056003cull, 0x3d006c0055003dull, 0x3e006c8055003eull, 0x35002300710035ull, 0x6a006c003f0039ull, 0x6a006c0040003aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c8059003cull, 0x3d00570075003dull, 0x3e006c8057003eull, 0x35002900720035ull, 0x39002700710039ull, 0x3a00280071003aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3c006c005a003cull, 0x3d006c0058003dull, 0x3e006c8058003eull, 0x35002f00730035ull, 0x39002d00720039ull, 0x3a002e0072003aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3d006c0059003dull, 0x6a006c003c0036ull, 0x6a006c003e0038ull, 0x39003300730039ull, 0x3a00340073003aull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36002400710036ull, 0x6a006c003d0037ull, 0x38002600710038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36002a00720036ull, 0x37002500710037ull, 0x38002c00720038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36003000730036ull, 0x37002b00720037ull, 0x38003200730038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x37003100730037ull, 0x36003580020036ull, 0x380035800d0038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x37003580070037ull, 0x380036800e0038ull, 0x39003680130039ull, 0x3a00368018003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x37003680080037ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x380037800f0038ull, 0x39003780140039ull, 0x3a00378019003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x39003880150039ull, 0x3a0038801a003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3a0039801b003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001c003a003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x39003a80170039ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001600390039ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x38003980110038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x38003a80120038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a001000380038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x370038800a0037ull, 0x35003880010035ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x370039800b0037ull, 0x6a000000350035ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x37003a800c0037ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000900370037ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36003780040036ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36003880050036ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36003a80060036ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a000300360036ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
};
constexpr int TLM_OPS = 1052;
static __device__ const double tlm_const_val[10] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 2.0};
static __device__ const unsigned long long tlm_prog[1052] = {
    0xb900b900b9009eull, 0xb900b900b9009full, 0xb900b900b900a0ull, 0xb900b900b900a1ull, 0xb900b900b900a2ull, 0xb900b900b900a3ull, 0xb900b900b900b0ull, 0xb800ba007800b2ull,
    0xb000ba00b200b0ull, 0xb800b0004700b0ull, 0xb800ba001f00b1ull, 0xb000b1007c00b0ull, 0xa000ba80b000a0ull, 0x9f00b000c1009full, 0xb900b900b900b0ull, 0xb80077001f00b2ull,
    0xb000ba00b200b0ull, 0xb80078001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0004800b0ull, 0xb8001f001e00b1ull, 0xb000b1007d00b0ull, 0x9f00ba80b0009full, 0xa000ba80b000a0ull,
    0xa100ba00b000a1ull, 0xb900b900b900b0ull, 0xb800ba007900b2ull, 0xb000ba00b200b0ull, 0xb800b0004900b0ull, 0xb800ba002000b1ull, 0xb000b1007e00b0ull, 0xa100ba80b000a1ull,
    0x9f00ba00b0009full, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb80077002000b2ull, 0xb000ba00b200b0ull, 0xb80079001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0004a00b0ull,
    0xb80020001e00b1ull, 0xb000b1007f00b0ull, 0x9f00ba80b0009full, 0xa100ba80b000a1ull, 0xa000b000c100a0ull, 0xb900b900b900b0ull, 0xb800ba007900b2ull, 0xb000ba00b200b0ull,
    0xb800b0004b00b0ull, 0xb800ba002000b1ull, 0xb000b1008000b0ull, 0xa100ba80b000a1ull, 0x9e00ba00b0009eull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ba007600b2ull,
    0xb000ba00b200b0ull, 0xb800b0004c00b0ull, 0xb800ba001d00b1ull, 0xb000b1008100b0ull, 0x9e00ba80b0009eull, 0x9f00ba00b0009full, 0xb900b900b900b0ull, 0xb80076002000b2ull,
    0xb000ba00b200b0ull, 0xb80079001d00b2ull, 0xb000ba00b200b0ull, 0xb800b0004d00b0ull, 0xb80020001d00b1ull, 0xb000b1008200b0ull, 0x9e00ba80b0009eull, 0xa100ba80b000a1ull,
    0xa000b000c100a0ull, 0xb900b900b900b0ull, 0xb80079002100b2ull, 0xb000ba00b200b0ull, 0xb8007a002000b2ull, 0xb000ba00b200b0ull, 0xb800b0004e00b0ull, 0xb80021002000b1ull,
    0xb000b1008300b0ull, 0xa200ba80b000a2ull, 0xa100ba80b000a1ull, 0xa300ba00b000a3ull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb80077002200b2ull, 0xb000ba00b200b0ull,
    0xb8007b001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0004f00b0ull, 0xb80022001e00b1ull, 0xb000b1008400b0ull, 0xa300ba80b000a3ull, 0x9f00ba80b0009full, 0xa200ba00b000a2ull,
    0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ba007b00b2ull, 0xb000ba00b200b0ull, 0xb800b0005000b0ull, 0xb800ba002200b1ull, 0xb000b1008500b0ull, 0xa300ba80b000a3ull,
    0xa200ba00b000a2ull, 0x9f00ba00b0009full, 0xb800ba009e0086ull, 0xb800ba009f0087ull, 0xb800ba00a00088ull, 0xb800ba00a10089ull, 0xb800ba00a2008aull, 0xb800ba00a3008bull,
    0xb900b900b900b0ull, 0xb800ba002500b2ull, 0xb000ba00b200b0ull, 0xb800b0007c00b0ull, 0xb900b900b900b1ull, 0xb000b1004700b0ull, 0x8800ba80b00088ull, 0x8700b000c10087ull,
    0xb900b900b900b0ull, 0xb80024001f00b2ull, 0xb000ba00b200b0ull, 0xb80025001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007d00b0ull, 0xb900b900b900b1ull, 0xb80078002400b2ull,
    0xb100ba00b200b1ull, 0xb80077002500b2ull, 0xb100ba00b200b1ull, 0xb000b1004800b0ull, 0x8700ba80b00087ull, 0x8800ba80b00088ull, 0x8900ba00b00089ull, 0xb900b900b900b0ull,
    0xb800ba002600b2ull, 0xb000ba00b200b0ull, 0xb800b0007e00b0ull, 0xb900b900b900b1ull, 0xb000b1004900b0ull, 0x8900ba80b00089ull, 0x8700ba00b00087ull, 0x8800ba00b00088ull,
    0xb900b900b900b0ull, 0xb80024002000b2ull, 0xb000ba00b200b0ull, 0xb80026001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007f00b0ull, 0xb900b900b900b1ull, 0xb80079002400b2ull,
    0xb100ba00b200b1ull, 0xb80077002600b2ull, 0xb100ba00b200b1ull, 0xb000b1004a00b0ull, 0x8700ba80b00087ull, 0x8900ba80b00089ull, 0x8800b000c10088ull, 0xb900b900b900b0ull,
    0xb800ba002600b2ull, 0xb000ba00b200b0ull, 0xb800b0008000b0ull, 0xb900b900b900b1ull, 0xb000b1004b00b0ull, 0x8900ba80b00089ull, 0x8600ba00b00086ull, 0x8800ba00b00088ull,
    0xb900b900b900b0ull, 0xb800ba002300b2ull, 0xb000ba00b200b0ull, 0xb800b0008100b0ull, 0xb900b900b900b1ull, 0xb000b1004c00b0ull, 0x8600ba80b00086ull, 0x8700ba00b00087ull,
    0xb900b900b900b0ull, 0xb80023002000b2ull, 0xb000ba00b200b0ull, 0xb80026001d00b2ull, 0xb000ba00b200b0ull, 0xb800b0008200b0ull, 0xb900b900b900b1ull, 0xb80079002300b2ull,
    0xb100ba00b200b1ull, 0xb80076002600b2ull, 0xb100ba00b200b1ull, 0xb000b1004d00b0ull, 0x8600ba80b00086ull, 0x8900ba80b00089ull, 0x8800b000c10088ull, 0xb900b900b900b0ull,
    0xb80026002100b2ull, 0xb000ba00b200b0ull, 0xb80027002000b2ull, 0xb000ba00b200b0ull, 0xb800b0008300b0ull, 0xb900b900b900b1ull, 0xb8007a002600b2ull, 0xb100ba00b200b1ull,
    0xb80079002700b2ull, 0xb100ba00b200b1ull, 0xb000b1004e00b0ull, 0x8a00ba80b0008aull, 0x8900ba80b00089ull, 0x8b00ba00b0008bull, 0x8800ba00b00088ull, 0xb900b900b900b0ull,
    0xb80024002200b2ull, 0xb000ba00b200b0ull, 0xb80028001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0008400b0ull, 0xb900b900b900b1ull, 0xb8007b002400b2ull, 0xb100ba00b200b1ull,
    0xb80077002800b2ull, 0xb100ba00b200b1ull, 0xb000b1004f00b0ull, 0x8b00ba80b0008bull, 0x8700ba80b00087ull, 0x8a00ba00b0008aull, 0x8800ba00b00088ull, 0xb900b900b900b0ull,
    0xb800ba002800b2ull, 0xb000ba00b200b0ull, 0xb800b0008500b0ull, 0xb900b900b900b1ull, 0xb000b1005000b0ull, 0x8b00ba80b0008bull, 0x8a00ba00b0008aull, 0x8700ba00b00087ull,
    0x87008680020087ull, 0x88008680070088ull, 0x88008780080088ull, 0x890086800d0089ull, 0x890087800e0089ull, 0x890088800f0089ull, 0x8a00878013008aull, 0x8a00888014008aull,
    0x8a00898015008aull, 0x8b00878018008bull, 0x8b00888019008bull, 0x8b0089801a008bull, 0x8b008a801b008bull, 0xb8001c008b008bull, 0x8a008b8017008aull, 0xb80016008a008aull,
    0x89008a80110089ull, 0x89008b80120089ull, 0xb8001000890089ull, 0x880089800a0088ull, 0x88008a800b0088ull, 0x88008b800c0088ull, 0xb8000900880088ull, 0x87008880040087ull,
    0x87008980050087ull, 0x87008b80060087ull, 0xb8000300870087ull, 0x86008980010086ull, 0xb8000000860086ull, 0xb800ba009e008cull, 0x8c008600bb008cull, 0xb800ba009f008dull,
    0x8d008700bb008dull, 0xb800ba00a0008eull, 0x8e008800bb008eull, 0xb800ba00a1008full, 0x8f008900bb008full, 0xb800ba00a20090ull, 0x90008a00bb0090ull, 0xb800ba00a30091ull,
    0x91008b00bb0091ull, 0xb900b900b900b0ull, 0xb800ba002b00b2ull, 0xb000ba00b200b0ull, 0xb800b0007c00b0ull, 0xb900b900b900b1ull, 0xb000b1004700b0ull, 0x8e00ba80b0008eull,
    0x8d00b000c1008dull, 0xb900b900b900b0ull, 0xb8002a001f00b2ull, 0xb000ba00b200b0ull, 0xb8002b001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007d00b0ull, 0xb900b900b900b1ull,
    0xb80078002a00b2ull, 0xb100ba00b200b1ull, 0xb80077002b00b2ull, 0xb100ba00b200b1ull, 0xb000b1004800b0ull, 0x8d00ba80b0008dull, 0x8e00ba80b0008eull, 0x8f00ba00b0008full,
    0xb900b900b900b0ull, 0xb800ba002c00b2ull, 0xb000ba00b200b0ull, 0xb800b0007e00b0ull, 0xb900b900b900b1ull, 0xb000b1004900b0ull, 0x8f00ba80b0008full, 0x8d00ba00b0008dull,
    0x8e00ba00b0008eull, 0xb900b900b900b0ull, 0xb8002a002000b2ull, 0xb000ba00b200b0ull, 0xb8002c001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007f00b0ull, 0xb900b900b900b1ull,
    0xb80079002a00b2ull, 0xb100ba00b200b1ull, 0xb80077002c00b2ull, 0xb100ba00b200b1ull, 0xb000b1004a00b0ull, 0x8d00ba80b0008dull, 0x8f00ba80b0008full, 0x8e00b000c1008eull,
    0xb900b900b900b0ull, 0xb800ba002c00b2ull, 0xb000ba00b200b0ull, 0xb800b0008000b0ull, 0xb900b900b900b1ull, 0xb000b1004b00b0ull, 0x8f00ba80b0008full, 0x8c00ba00b0008cull,
    0x8e00ba00b0008eull, 0xb900b900b900b0ull, 0xb800ba002900b2ull, 0xb000ba00b200b0ull, 0xb800b0008100b0ull, 0xb900b900b900b1ull, 0xb000b1004c00b0ull, 0x8c00ba80b0008cull,
    0x8d00ba00b0008dull, 0xb900b900b900b0ull, 0xb80029002000b2ull, 0xb000ba00b200b0ull, 0xb8002c001d00b2ull, 0xb000ba00b200b0ull, 0xb800b0008200b0ull, 0xb900b900b900b1ull,
    0xb80079002900b2ull, 0xb100ba00b200b1ull, 0xb80076002c00b2ull, 0xb100ba00b200b1ull, 0xb000b1004d00b0ull, 0x8c00ba80b0008cull, 0x8f00ba80b0008full, 0x8e00b000c1008eull,
    0xb900b900b900b0ull, 0xb8002c002100b2ull, 0xb000ba00b200b0ull, 0xb8002d002000b2ull, 0xb000ba00b200b0ull, 0xb800b0008300b0ull, 0xb900b900b900b1ull, 0xb8007a002c00b2ull,
    0xb100ba00b200b1ull, 0xb80079002d00b2ull, 0xb100ba00b200b1ull, 0xb000b1004e00b0ull, 0x9000ba80b00090ull, 0x8f00ba80b0008full, 0x9100ba00b00091ull, 0x8e00ba00b0008eull,
    0xb900b900b900b0ull, 0xb8002a002200b2ull, 0xb000ba00b200b0ull, 0xb8002e001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0008400b0ull, 0xb900b900b900b1ull, 0xb8007b002a00b2ull,
    0xb100ba00b200b1ull, 0xb80077002e00b2ull, 0xb100ba00b200b1ull, 0xb000b1004f00b0ull, 0x9100ba80b00091ull, 0x8d00ba80b0008dull, 0x9000ba00b00090ull, 0x8e00ba00b0008eull,
    0xb900b900b900b0ull, 0xb800ba002e00b2ull, 0xb000ba00b200b0ull, 0xb800b0008500b0ull, 0xb900b900b900b1ull, 0xb000b1005000b0ull, 0x9100ba80b00091ull, 0x9000ba00b00090ull,
    0x8d00ba00b0008dull, 0x8d008c8002008dull, 0x8e008c8007008eull, 0x8e008d8008008eull, 0x8f008c800d008full, 0x8f008d800e008full, 0x8f008e800f008full, 0x90008d80130090ull,
    0x90008e80140090ull, 0x90008f80150090ull, 0x91008d80180091ull, 0x91008e80190091ull, 0x91008f801a0091ull, 0x910090801b0091ull, 0xb8001c00910091ull, 0x90009180170090ull,
    0xb8001600900090ull, 0x8f00908011008full, 0x8f00918012008full, 0xb80010008f008full, 0x8e008f800a008eull, 0x8e0090800b008eull, 0x8e0091800c008eull, 0xb80009008e008eull,
    0x8d008e8004008dull, 0x8d008f8005008dull, 0x8d00918006008dull, 0xb80003008d008dull, 0x8c008f8001008cull, 0xb80000008c008cull, 0xb800ba001d00a4ull, 0xb800ba007600aaull,
    0xa4002300c100a4ull, 0xaa008600c100aaull, 0xb800ba001e00a5ull, 0xb800ba007700abull, 0xa5002400c100a5ull, 0xab008700c100abull, 0xb800ba001f00a6ull, 0xb800ba007800acull,
    0xa6002500c100a6ull, 0xac008800c100acull, 0xb800ba002000a7ull, 0xb800ba007900adull, 0xa7002600c100a7ull, 0xad008900c100adull, 0xb800ba002100a8ull, 0xb800ba007a00aeull,
    0xa8002700c100a8ull, 0xae008a00c100aeull, 0xb800ba002200a9ull, 0xb800ba007b00afull, 0xa9002800c100a9ull, 0xaf008b00c100afull, 0xb900b900b9009eull, 0xb900b900b9009full,
    0xb900b900b900a0ull, 0xb900b900b900a1ull, 0xb900b900b900a2ull, 0xb900b900b900a3ull, 0xb900b900b900b0ull, 0xb800ba00ac00b2ull, 0xb000ba00b200b0ull, 0xb800b0004700b0ull,
    0xb800ba00a600b1ull, 0xb000b1007c00b0ull, 0xa000ba80b000a0ull, 0x9f00b000c1009full, 0xb900b900b900b0ull, 0xb800ab00a600b2ull, 0xb000ba00b200b0ull, 0xb800ac00a500b2ull,
    0xb000ba00b200b0ull, 0xb800b0004800b0ull, 0xb800a600a500b1ull, 0xb000b1007d00b0ull, 0x9f00ba80b0009full, 0xa000ba80b000a0ull, 0xa100ba00b000a1ull, 0xb900b900b900b0ull,
    0xb800ba00ad00b2ull, 0xb000ba00b200b0ull, 0xb800b0004900b0ull, 0xb800ba00a700b1ull, 0xb000b1007e00b0ull, 0xa100ba80b000a1ull, 0x9f00ba00b0009full, 0xa000ba00b000a0ull,
    0xb900b900b900b0ull, 0xb800ab00a700b2ull, 0xb000ba00b200b0ull, 0xb800ad00a500b2ull, 0xb000ba00b200b0ull, 0xb800b0004a00b0ull, 0xb800a700a500b1ull, 0xb000b1007f00b0ull,
    0x9f00ba80b0009full, 0xa100ba80b000a1ull, 0xa000b000c100a0ull, 0xb900b900b900b0ull, 0xb800ba00ad00b2ull, 0xb000ba00b200b0ull, 0xb800b0004b00b0ull, 0xb800ba00a700b1ull,
    0xb000b1008000b0ull, 0xa100ba80b000a1ull, 0x9e00ba00b0009eull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ba00aa00b2ull, 0xb000ba00b200b0ull, 0xb800b0004c00b0ull,
    0xb800ba00a400b1ull, 0xb000b1008100b0ull, 0x9e00ba80b0009eull, 0x9f00ba00b0009full, 0xb900b900b900b0ull, 0xb800aa00a700b2ull, 0xb000ba00b200b0ull, 0xb800ad00a400b2ull,
    0xb000ba00b200b0ull, 0xb800b0004d00b0ull, 0xb800a700a400b1ull, 0xb000b1008200b0ull, 0x9e00ba80b0009eull, 0xa100ba80b000a1ull, 0xa000b000c100a0ull, 0xb900b900b900b0ull,
    0xb800ad00a800b2ull, 0xb000ba00b200b0ull, 0xb800ae00a700b2ull, 0xb000ba00b200b0ull, 0xb800b0004e00b0ull, 0xb800a800a700b1ull, 0xb000b1008300b0ull, 0xa200ba80b000a2ull,
    0xa100ba80b000a1ull, 0xa300ba00b000a3ull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ab00a900b2ull, 0xb000ba00b200b0ull, 0xb800af00a500b2ull, 0xb000ba00b200b0ull,
    0xb800b0004f00b0ull, 0xb800a900a500b1ull, 0xb000b1008400b0ull, 0xa300ba80b000a3ull, 0x9f00ba80b0009full, 0xa200ba00b000a2ull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull,
    0xb800ba00af00b2ull, 0xb000ba00b200b0ull, 0xb800b0005000b0ull, 0xb800ba00a900b1ull, 0xb000b1008500b0ull, 0xa300ba80b000a3ull, 0xa200ba00b000a2ull, 0x9f00ba00b0009full,
    0xb800ba009e0092ull, 0x92008600bc0092ull, 0x92008c00bd0092ull, 0xb800ba009f0093ull, 0x93008700bc0093ull, 0x93008d00bd0093ull, 0xb800ba00a00094ull, 0x94008800bc0094ull,
    0x94008e00bd0094ull, 0xb800ba00a10095ull, 0x95008900bc0095ull, 0x95008f00bd0095ull, 0xb800ba00a20096ull, 0x96008a00bc0096ull, 0x96009000bd0096ull, 0xb800ba00a30097ull,
    0x97008b00bc0097ull, 0x97009100bd0097ull, 0xb900b900b900b0ull, 0xb800ba003100b2ull, 0xb000ba00b200b0ull, 0xb800b0007c00b0ull, 0xb900b900b900b1ull, 0xb000b1004700b0ull,
    0x9400ba80b00094ull, 0x9300b000c10093ull, 0xb900b900b900b0ull, 0xb80030001f00b2ull, 0xb000ba00b200b0ull, 0xb80031001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007d00b0ull,
    0xb900b900b900b1ull, 0xb80078003000b2ull, 0xb100ba00b200b1ull, 0xb80077003100b2ull, 0xb100ba00b200b1ull, 0xb000b1004800b0ull, 0x9300ba80b00093ull, 0x9400ba80b00094ull,
    0x9500ba00b00095ull, 0xb900b900b900b0ull, 0xb800ba003200b2ull, 0xb000ba00b200b0ull, 0xb800b0007e00b0ull, 0xb900b900b900b1ull, 0xb000b1004900b0ull, 0x9500ba80b00095ull,
    0x9300ba00b00093ull, 0x9400ba00b00094ull, 0xb900b900b900b0ull, 0xb80030002000b2ull, 0xb000ba00b200b0ull, 0xb80032001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007f00b0ull,
    0xb900b900b900b1ull, 0xb80079003000b2ull, 0xb100ba00b200b1ull, 0xb80077003200b2ull, 0xb100ba00b200b1ull, 0xb000b1004a00b0ull, 0x9300ba80b00093ull, 0x9500ba80b00095ull,
    0x9400b000c10094ull, 0xb900b900b900b0ull, 0xb800ba003200b2ull, 0xb000ba00b200b0ull, 0xb800b0008000b0ull, 0xb900b900b900b1ull, 0xb000b1004b00b0ull, 0x9500ba80b00095ull,
    0x9200ba00b00092ull, 0x9400ba00b00094ull, 0xb900b900b900b0ull, 0xb800ba002f00b2ull, 0xb000ba00b200b0ull, 0xb800b0008100b0ull, 0xb900b900b900b1ull, 0xb000b1004c00b0ull,
    0x9200ba80b00092ull, 0x9300ba00b00093ull, 0xb900b900b900b0ull, 0xb8002f002000b2ull, 0xb000ba00b200b0ull, 0xb80032001d00b2ull, 0xb000ba00b200b0ull, 0xb800b0008200b0ull,
    0xb900b900b900b1ull, 0xb80079002f00b2ull, 0xb100ba00b200b1ull, 0xb80076003200b2ull, 0xb100ba00b200b1ull, 0xb000b1004d00b0ull, 0x9200ba80b00092ull, 0x9500ba80b00095ull,
    0x9400b000c10094ull, 0xb900b900b900b0ull, 0xb80032002100b2ull, 0xb000ba00b200b0ull, 0xb80033002000b2ull, 0xb000ba00b200b0ull, 0xb800b0008300b0ull, 0xb900b900b900b1ull,
    0xb8007a003200b2ull, 0xb100ba00b200b1ull, 0xb80079003300b2ull, 0xb100ba00b200b1ull, 0xb000b1004e00b0ull, 0x9600ba80b00096ull, 0x9500ba80b00095ull, 0x9700ba00b00097ull,
    0x9400ba00b00094ull, 0xb900b900b900b0ull, 0xb80030002200b2ull, 0xb000ba00b200b0ull, 0xb80034001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0008400b0ull, 0xb900b900b900b1ull,
    0xb8007b003000b2ull, 0xb100ba00b200b1ull, 0xb80077003400b2ull, 0xb100ba00b200b1ull, 0xb000b1004f00b0ull, 0x9700ba80b00097ull, 0x9300ba80b00093ull, 0x9600ba00b00096ull,
    0x9400ba00b00094ull, 0xb900b900b900b0ull, 0xb800ba003400b2ull, 0xb000ba00b200b0ull, 0xb800b0008500b0ull, 0xb900b900b900b1ull, 0xb000b1005000b0ull, 0x9700ba80b00097ull,
    0x9600ba00b00096ull, 0x9300ba00b00093ull, 0x93009280020093ull, 0x94009280070094ull, 0x94009380080094ull, 0x950092800d0095ull, 0x950093800e0095ull, 0x950094800f0095ull,
    0x96009380130096ull, 0x96009480140096ull, 0x96009580150096ull, 0x97009380180097ull, 0x97009480190097ull, 0x970095801a0097ull, 0x970096801b0097ull, 0xb8001c00970097ull,
    0x96009780170096ull, 0xb8001600960096ull, 0x95009680110095ull, 0x95009780120095ull, 0xb8001000950095ull, 0x940095800a0094ull, 0x940096800b0094ull, 0x940097800c0094ull,
    0xb8000900940094ull, 0x93009480040093ull, 0x93009580050093ull, 0x93009780060093ull, 0xb8000300930093ull, 0x92009580010092ull, 0xb8000000920092ull, 0xb800ba001d00a4ull,
    0xb800ba007600aaull, 0xa4002300c100a4ull, 0xaa008600c100aaull, 0xa400ba002f00a4ull, 0xaa00ba009200aaull, 0xb800ba001e00a5ull, 0xb800ba007700abull, 0xa5002400c100a5ull,
    0xab008700c100abull, 0xa500ba003000a5ull, 0xab00ba009300abull, 0xb800ba001f00a6ull, 0xb800ba007800acull, 0xa6002500c100a6ull, 0xac008800c100acull, 0xa600ba003100a6ull,
    0xac00ba009400acull, 0xb800ba002000a7ull, 0xb800ba007900adull, 0xa7002600c100a7ull, 0xad008900c100adull, 0xa700ba003200a7ull, 0xad00ba009500adull, 0xb800ba002100a8ull,
    0xb800ba007a00aeull, 0xa8002700c100a8ull, 0xae008a00c100aeull, 0xa800ba003300a8ull, 0xae00ba009600aeull, 0xb800ba002200a9ull, 0xb800ba007b00afull, 0xa9002800c100a9ull,
    0xaf008b00c100afull, 0xa900ba003400a9ull, 0xaf00ba009700afull, 0xb900b900b9009eull, 0xb900b900b9009full, 0xb900b900b900a0ull, 0xb900b900b900a1ull, 0xb900b900b900a2ull,
    0xb900b900b900a3ull, 0xb900b900b900b0ull, 0xb800ba00ac00b2ull, 0xb000ba00b200b0ull, 0xb800b0004700b0ull, 0xb800ba00a600b1ull, 0xb000b1007c00b0ull, 0xa000ba80b000a0ull,
    0x9f00b000c1009full, 0xb900b900b900b0ull, 0xb800ab00a600b2ull, 0xb000ba00b200b0ull, 0xb800ac00a500b2ull, 0xb000ba00b200b0ull, 0xb800b0004800b0ull, 0xb800a600a500b1ull,
    0xb000b1007d00b0ull, 0x9f00ba80b0009full, 0xa000ba80b000a0ull, 0xa100ba00b000a1ull, 0xb900b900b900b0ull, 0xb800ba00ad00b2ull, 0xb000ba00b200b0ull, 0xb800b0004900b0ull,
    0xb800ba00a700b1ull, 0xb000b1007e00b0ull, 0xa100ba80b000a1ull, 0x9f00ba00b0009full, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ab00a700b2ull, 0xb000ba00b200b0ull,
    0xb800ad00a500b2ull, 0xb000ba00b200b0ull, 0xb800b0004a00b0ull, 0xb800a700a500b1ull, 0xb000b1007f00b0ull, 0x9f00ba80b0009full, 0xa100ba80b000a1ull, 0xa000b000c100a0ull,
    0xb900b900b900b0ull, 0xb800ba00ad00b2ull, 0xb000ba00b200b0ull, 0xb800b0004b00b0ull, 0xb800ba00a700b1ull, 0xb000b1008000b0ull, 0xa100ba80b000a1ull, 0x9e00ba00b0009eull,
    0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ba00aa00b2ull, 0xb000ba00b200b0ull, 0xb800b0004c00b0ull, 0xb800ba00a400b1ull, 0xb000b1008100b0ull, 0x9e00ba80b0009eull,
    0x9f00ba00b0009full, 0xb900b900b900b0ull, 0xb800aa00a700b2ull, 0xb000ba00b200b0ull, 0xb800ad00a400b2ull, 0xb000ba00b200b0ull, 0xb800b0004d00b0ull, 0xb800a700a400b1ull,
    0xb000b1008200b0ull, 0x9e00ba80b0009eull, 0xa100ba80b000a1ull, 0xa000b000c100a0ull, 0xb900b900b900b0ull, 0xb800ad00a800b2ull, 0xb000ba00b200b0ull, 0xb800ae00a700b2ull,
    0xb000ba00b200b0ull, 0xb800b0004e00b0ull, 0xb800a800a700b1ull, 0xb000b1008300b0ull, 0xa200ba80b000a2ull, 0xa100ba80b000a1ull, 0xa300ba00b000a3ull, 0xa000ba00b000a0ull,
    0xb900b900b900b0ull, 0xb800ab00a900b2ull, 0xb000ba00b200b0ull, 0xb800af00a500b2ull, 0xb000ba00b200b0ull, 0xb800b0004f00b0ull, 0xb800a900a500b1ull, 0xb000b1008400b0ull,
    0xa300ba80b000a3ull, 0x9f00ba80b0009full, 0xa200ba00b000a2ull, 0xa000ba00b000a0ull, 0xb900b900b900b0ull, 0xb800ba00af00b2ull, 0xb000ba00b200b0ull, 0xb800b0005000b0ull,
    0xb800ba00a900b1ull, 0xb000b1008500b0ull, 0xa300ba80b000a3ull, 0xa200ba00b000a2ull, 0x9f00ba00b0009full, 0xb800ba009e0098ull, 0x98008600be0098ull, 0x98008c00bf0098ull,
    0x98009200c00098ull, 0xb800ba009f0099ull, 0x99008700be0099ull, 0x99008d00bf0099ull, 0x99009300c00099ull, 0xb800ba00a0009aull, 0x9a008800be009aull, 0x9a008e00bf009aull,
    0x9a009400c0009aull, 0xb800ba00a1009bull, 0x9b008900be009bull, 0x9b008f00bf009bull, 0x9b009500c0009bull, 0xb800ba00a2009cull, 0x9c008a00be009cull, 0x9c009000bf009cull,
    0x9c009600c0009cull, 0xb800ba00a3009dull, 0x9d008b00be009dull, 0x9d009100bf009dull, 0x9d009700c0009dull, 0xb900b900b900b0ull, 0xb800ba003700b2ull, 0xb000ba00b200b0ull,
    0xb800b0007c00b0ull, 0xb900b900b900b1ull, 0xb000b1004700b0ull, 0x9a00ba80b0009aull, 0x9900b000c10099ull, 0xb900b900b900b0ull, 0xb80036001f00b2ull, 0xb000ba00b200b0ull,
    0xb80037001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007d00b0ull, 0xb900b900b900b1ull, 0xb80078003600b2ull, 0xb100ba00b200b1ull, 0xb80077003700b2ull, 0xb100ba00b200b1ull,
    0xb000b1004800b0ull, 0x9900ba80b00099ull, 0x9a00ba80b0009aull, 0x9b00ba00b0009bull, 0xb900b900b900b0ull, 0xb800ba003800b2ull, 0xb000ba00b200b0ull, 0xb800b0007e00b0ull,
    0xb900b900b900b1ull, 0xb000b1004900b0ull, 0x9b00ba80b0009bull, 0x9900ba00b00099ull, 0x9a00ba00b0009aull, 0xb900b900b900b0ull, 0xb80036002000b2ull, 0xb000ba00b200b0ull,
    0xb80038001e00b2ull, 0xb000ba00b200b0ull, 0xb800b0007f00b0ull, 0xb900b900b900b1ull, 0xb80079003600b2ull, 0xb100ba00b200b1ull, 0xb80077003800b2ull, 0xb100ba00b200b1ull,
    0xb000b1004a00b0ull, 0x9900ba80b00099ull, 0x9b00ba80b0009bull, 0x9a00b000c1009aull, 0xb900b900b900b0ull, 0xb800ba003800b2ull, 0xb000ba00b200b0ull, 0xb800b0008000b0ull,
    0xb900b900b900b1ull, 0xb000b1004b00b0ull, 0x9b00ba80b0009bull, 0x9800ba00b00098ull, 0x9a00ba00b0009aull, 0xb900b900b900b0ull, 0xb800ba003500b2ull, 0xb000ba00b200b0ull,
    0xb800b0008100b0ull, 0xb900b900b900b1ull, 0xb000b1004c00b0ull, 0x9800ba80b00098ull, 0x9900ba00b00099ull, 0xb900b900b900b0ull, 0xb80035002000b2ull, 0xb000ba00b200b0ull,
    0xb80038001d00b2ull, 0xb000ba00b200b0ull, 0xb800b0008200b0ull, 0xb900b900b900b1ull, 0xb80079003500b2ull, 0xb100ba00b200b1ull, 0xb80076003800b2ull, 0xb100ba00b200b1ull,
    0xb000b1004d00b0ull, 0x9800ba80b00098ull, 0x9b00ba80b0009bull, 0x9a00b000c1009aull, 0xb900b900b900b0ull, 0xb80038002100b2ull, 0xb000ba00b200b0ull, 0xb80039002000b2ull,
    0xb000ba00b200b0ull, 0xb800b0008300b0ull, 0xb900b900b900b1ull, 0xb8007a003800b2ull, 0xb100ba00b200b1ull, 0xb80079003900b2ull, 0xb100ba00b200b1ull, 0xb000b1004e00b0ull,
    0x9c00ba80b0009cull, 0x9b00ba80b0009bull, 0x9d00ba00b0009dull, 0x9a00ba00b0009aull, 0xb900b900b900b0ull, 0xb80036002200b2ull, 0xb000ba00b200b0ull, 0xb8003a001e00b2ull,
    0xb000ba00b200b0ull, 0xb800b0008400b0ull, 0xb900b900b900b1ull, 0xb8007b003600b2ull, 0xb100ba00b200b1ull, 0xb80077003a00b2ull, 0xb100ba00b200b1ull, 0xb000b1004f00b0ull,
    0x9d00ba80b0009dull, 0x9900ba80b00099ull, 0x9c00ba00b0009cull, 0x9a00ba00b0009aull, 0xb900b900b900b0ull, 0xb800ba003a00b2ull, 0xb000ba00b200b0ull, 0xb800b0008500b0ull,
    0xb900b900b900b1ull, 0xb000b1005000b0ull, 0x9d00ba80b0009dull, 0x9c00ba00b0009cull, 0x9900ba00b00099ull, 0x99009880020099ull, 0x9a00988007009aull, 0x9a00998008009aull,
    0x9b0098800d009bull, 0x9b0099800e009bull, 0x9b009a800f009bull, 0x9c00998013009cull, 0x9c009a8014009cull, 0x9c009b8015009cull, 0x9d00998018009dull, 0x9d009a8019009dull,
    0x9d009b801a009dull, 0x9d009c801b009dull, 0xb8001c009d009dull, 0x9c009d8017009cull, 0xb80016009c009cull, 0x9b009c8011009bull, 0x9b009d8012009bull, 0xb80010009b009bull,
    0x9a009b800a009aull, 0x9a009c800b009aull, 0x9a009d800c009aull, 0xb80009009a009aull, 0x99009a80040099ull, 0x99009b80050099ull, 0x99009d80060099ull, 0xb8000300990099ull,
    0x98009b80010098ull, 0xb8000000980098ull, 0x76008600c10076ull, 0x7600ba00920076ull, 0x7600ba00980076ull, 0x77008700c10077ull, 0x7700ba00930077ull, 0x7700ba00990077ull,
    0x78008800c10078ull, 0x7800ba00940078ull, 0x7800ba009a0078ull, 0x79008900c10079ull, 0x7900ba00950079ull, 0x7900ba009b0079ull, 0x7a008a00c1007aull, 0x7a00ba0096007aull,
    0x7a00ba009c007aull, 0x7b008b00c1007bull, 0x7b00ba0097007bull, 0x7b00ba009d007bull,
};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "small_strato_rodas3";
  static constexpr int NS = 7;      // species including fixed ones
  static constexpr int NV = 6;      // variable species (solved system)
  static constexpr int NR = 10;      // reactions
  static constexpr int NP = 4;      // runtime parameter slots per cell
  static constexpr int NPH = 4;      // photolysis slots
  static constexpr int NFIX = 1;
  static constexpr int NLU = 29;
  static constexpr int NSTAGE = 4;
  static constexpr bool RUNTIME_ENV = false;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.5;
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
  static constexpr double ATOL[NS] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
  static constexpr double RTOL[NS] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001};
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
  static constexpr int F = 59;
  static constexpr int DY = 65;
  static constexpr int KT = 71;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 81;
  static constexpr bool TABLE_ATTEMPT = false;

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
    const double c21 = 4.0 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[41 + i] = fma(c21, S[35 + i], S[F + i]);
    }
    solve(S, 41);
    fun([&](int i) { return S[Y + i] + 2.0 * S[35 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c31 = 1.0 / h;
    const double c32 = -1.0 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[47 + i] = fma(c32, S[41 + i], fma(c31, S[35 + i], S[F + i]));
    }
    solve(S, 47);
    fun([&](int i) { return S[Y + i] + 2.0 * S[35 + i] + S[47 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c41 = 1.0 / h;
    const double c42 = -1.0 / h;
    const double c43 = -2.6666666666666665 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[53 + i] = fma(c43, S[47 + i], fma(c42, S[41 + i], fma(c41, S[35 + i], S[F + i])));
    }
    solve(S, 53);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[35 + i];
      const double k1 = S[41 + i];
      const double k2 = S[47 + i];
      const double k3 = S[53 + i];
      const double yi = S[Y + i];
      const double ynew = fma(2.0, k0, yi) + k2 + k3;
      S[DY + i] = 2.0 * k0 + k2 + k3;
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (k3) / sc;
      err_sq = fma(q, q, err_sq);
    }
    return fmax(sqrt(err_sq / 7.0), 1.0e-10);
  }

  // Step-size factor from the error norm (integrate.j2:324-333).
  __device__ __forceinline__ static double growth(double err) {
    const double fac = 0.9 / cbrt(err);
    return fmax(0.2, fmin(fac, 6.0));
  }

  // ---- warp-cooperative attempt (static warp schedules) ----
  static constexpr int NPART = 15;
  static constexpr int Q = 81;            // rates q_r, then q_i of the error norm
  static constexpr int D = 91;     // partial derivatives
  static constexpr int CB = 106;        // constants
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
      S[110] = 4.0 / h;    // c21 / h
      S[111] = 1.0 / h;    // c31 / h
      S[112] = -1.0 / h;    // c32 / h
      S[113] = 1.0 / h;    // c41 / h
      S[114] = -1.0 / h;    // c42 / h
      S[115] = -2.6666666666666665 / h;    // c43 / h
    }
    __syncwarp();
    bool ok = true;
    for (int st = 0; st < NSTAGE; ++st) ok = run_schedule(S, T::stage_step[st], T::stage_step[st + 1], lane) && ok;
    if (__any_sync(0xffffffffu, !ok)) status |= 1;
    // Increment, and q_i^2 of the error norm into the rate slots.
    for (int i = lane; i < NV; i += 32) {
      const double k0 = S[35 + i];
      const double k1 = S[41 + i];
      const double k2 = S[47 + i];
      const double k3 = S[53 + i];
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
      err = fmax(sqrt(err_sq / 7.0), 1.0e-10);
    }
    return __shfl_sync(0xffffffffu, err, 0);
  }

  // ---- tangent of one accepted step (forward sensitivities) ----
  static constexpr int DYT = 118;     // dy in, dy_new out (NV)
  static constexpr int DKR = 124;     // dk, the rate constants' tangent (NR)
  static constexpr int TLM_CB = 184;  // constants of the tangent program
  static constexpr int TLM_NCONST = 10;
  static constexpr int NSLOTS_TLM = 194;
  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks
  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and
  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].
  template <class SA, class KA>
  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {
    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);
    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];
    S[187] = 4.0 / h;    // c21 / h
    S[188] = 1.0 / h;    // c31 / h
    S[189] = -1.0 / h;    // c32 / h
    S[190] = 1.0 / h;    // c41 / h
    S[191] = -1.0 / h;    // c42 / h
    S[192] = -2.6666666666666665 / h;    // c43 / h
    for (int n = 0; n < coop::TLM_OPS; ++n) {
      const unsigned long long w = __ldg(coop::tlm_prog + n);
      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                            ((long long)(lo >> 31) << 63));
      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
    }
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 81;      // dL/dy
  static constexpr int KBAR = 87;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 111;    // adjoint of the pending stage tendency
  static constexpr int KB = 117;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 127;
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
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 2.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 6 + j] = 0.0;
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 12 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 18 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 4
    solve_t(S, KBAR + 18);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 18, 53);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 18 + j];
    { const double cc = 1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 18 + q], S[KBAR + 0 + q]); }
    { const double cc = -1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 6 + q] = fma(cc, S[KBAR + 18 + q], S[KBAR + 6 + q]); }
    { const double cc = -2.6666666666666665 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 12 + q] = fma(cc, S[KBAR + 18 + q], S[KBAR + 12 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + 2.0 * S[35 + q] + S[47 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(2.0, x, S[KBAR + 0 + j]); S[KBAR + 12 + j] = fma(1.0, x, S[KBAR + 12 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 12);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 12, 47);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 12 + j];
    { const double cc = 1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 12 + q], S[KBAR + 0 + q]); }
    { const double cc = -1.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 6 + q] = fma(cc, S[KBAR + 12 + q], S[KBAR + 6 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + 2.0 * S[35 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(2.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 2
    solve_t(S, KBAR + 6);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 6, 41);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 6 + j];
    { const double cc = 4.0 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 6 + q], S[KBAR + 0 + q]); }
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

}  // namespace mkpp_small_strato_rodas3
