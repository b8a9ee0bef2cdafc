// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/small_strato.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 7 species (6 variable), 10 reactions, 26 W slots, 29 LU slots, 29 LU products, 13 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_small_strato {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const double const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, -2.0, 2.0};
static __device__ const int stage_step[4] = {0, 31, 62, 84};
static __device__ const unsigned long long sched[2688] = {
    0x64006600410055ull, 0x64001f00420056ull, 0x64001e00420057ull, 0x64006600430058ull, 0x64002000440059ull, 0x64001e0044005aull, 0x6400660045005bull, 0x6400660046005cull,
    0x6400200047005dull, 0x64001d0047005eull, 0x6400200048005full, 0x64002100480060ull, 0x64001e00490061ull, 0x64002200490062ull, 0x640066004a0063ull, 0x65006500650014ull,
    0x65006500650019ull, 0x65006500650012ull, 0x64001f0041004bull, 0x64001e0042004cull, 0x6400200043004dull, 0x64001e0044004eull, 0x6400200045004full, 0x64001d00460050ull,
    0x64001d00470051ull, 0x64002100480052ull, 0x64002200490053ull, 0x640022004a0054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x670066005c0000ull, 0x640066805b0001ull, 0x640066805c0002ull, 0x67006600560003ull, 0x64006b00550004ull, 0x64006680580005ull, 0x64006600610006ull, 0x64006b005d0007ull,
    0x64006600560008ull, 0x67006600550009ull, 0x6400668058000aull, 0x640066805f000bull, 0x640066005d000dull, 0x6400668056000eull, 0x6400668057000full, 0x67006600580010ull,
    0x640066005f0011ull, 0x64006680620013ull, 0x64006600600015ull, 0x670066005f0016ull, 0x64006680610017ull, 0x64006600620018ull, 0x6400668060001aull, 0x6700660061001cull,
    0x64001f004c004cull, 0x640020004e004eull, 0x64002000510051ull, 0x64002000520052ull, 0x64001e00530053ull, 0x640066004f0035ull, 0x64006c004b0036ull, 0x640066804b0037ull,
    0x66005d0000ull, 0x10066005e0001ull, 0x3006600590003ull, 0x4006600570004ull, 0x50066005a0005ull, 0x6006680630006ull, 0x80059006b0008ull, 0x9006600570009ull,
    0xa005a006b000aull, 0x6400668061000cull, 0xe00660059000eull, 0x100066005a0010ull, 0x17006680630017ull, 0x640066805f001bull, 0x1c00660063001cull, 0x35006680500035ull,
    0x360066804c0036ull, 0x370066804c0037ull, 0x640066004c0038ull, 0x64006680520039ull, 0x6400660052003aull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3006600620003ull, 0x8006680620008ull, 0xa0066805b000aull, 0x100066005b0010ull, 0x8000000000000000ull, 0x35006680510035ull, 0x360066004d0036ull, 0x370066004d0037ull,
    0x380066804d0038ull, 0x39006600530039ull, 0x3a00668053003aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xa005e006b000aull, 0x100066005e0010ull, 0x64000000020002ull, 0x64000000070007ull, 0x640000000d000dull, 0x8000000000000003ull, 0x360066804e0036ull, 0x37004e006c0037ull,
    0x380066804e0038ull, 0x39006600540039ull, 0x3a00668054003aull, 0x64006600350023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xa00668060000aull, 0x10006600600010ull, 0x5000180020005ull, 0x64000300080008ull, 0x640003000e000eull, 0x64000300130013ull, 0x64000300180018ull, 0x36006600500036ull,
    0x370066004f0037ull, 0x380066804f0038ull, 0x64006600390027ull, 0x640066003a0028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x9000480080009ull, 0xa00018007000aull, 0xc00068008000cull, 0xf0004800e000full, 0x14000480130014ull, 0x19000480180019ull, 0x100001800d0010ull, 0x120006800e0012ull,
    0x15000580130015ull, 0x1a00058018001aull, 0x17000680130017ull, 0x1c00068018001cull, 0x36006680530036ull, 0x370051006c0037ull, 0x38006680510038ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000009ull, 0xa00058008000aull, 0x100005800e0010ull, 0x36006600540036ull, 0x37006600520037ull, 0x38006680520038ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x640009000f000full, 0x64000900140014ull, 0x64000900190019ull, 0x37006600530037ull, 0x64006600360024ull, 0x64006600380026ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x10000a800f0010ull, 0x11000b800f0011ull, 0x12000c800f0012ull, 0x15000a80140015ull, 0x1a000a8019001aull, 0x16000b80140016ull, 0x17000c80140017ull, 0x1b000b8019001bull,
    0x1c000c8019001cull, 0x64006600370025ull, 0x24002380020024ull, 0x260023800d0026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000010ull, 0x25002380070025ull, 0x260024800e0026ull, 0x27002480130027ull, 0x28002480180028ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64001000150015ull, 0x640010001a001aull, 0x25002480080025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x640016001b001bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64001c00280028ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x27002880170027ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64001600270027ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64001000260026ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250026800a0025ull, 0x23002680010023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250027800b0025ull, 0x64000000230023ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x250028800c0025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64000900250025ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64000300240024ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x1d00660023003bull, 0x1e00660024003cull, 0x1f00660025003dull, 0x2000660026003eull, 0x2100660027003full, 0x22006600280040ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64003d0041004bull, 0x64003c0042004cull, 0x64003e0043004dull, 0x64003c0044004eull, 0x64003e0045004full, 0x64003b00460050ull, 0x64003b00470051ull, 0x64003f00480052ull,
    0x64004000490053ull, 0x640040004a0054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64003d004c004cull, 0x64003e004e004eull, 0x64003e00510051ull, 0x64003e00520052ull, 0x64003c00530053ull, 0x640066004f0035ull, 0x64006c004b0036ull, 0x640066804b0037ull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x35006680500035ull, 0x360066804c0036ull, 0x370066804c0037ull, 0x640066004c0038ull, 0x64006680520039ull, 0x6400660052003aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x35006680510035ull, 0x360066004d0036ull, 0x370066004d0037ull, 0x380066804d0038ull, 0x39006600530039ull, 0x3a00668053003aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x360066804e0036ull, 0x37004e006c0037ull, 0x380066804e0038ull, 0x39006600540039ull, 0x3a00668054003aull, 0x64006600350029ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36006600500036ull, 0x370066004f0037ull, 0x380066804f0038ull, 0x29002300680029ull, 0x6400660039002dull, 0x640066003a002eull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36006680530036ull, 0x370051006c0037ull, 0x38006680510038ull, 0x2d00270068002dull, 0x2e00280068002eull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x36006600540036ull, 0x37006600520037ull, 0x38006680520038ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x37006600530037ull, 0x6400660036002aull, 0x6400660038002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2a00240068002aull, 0x6400660037002bull, 0x2c00260068002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b00250068002bull, 0x2a00298002002aull, 0x2c0029800d002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b00298007002bull, 0x2c002a800e002cull, 0x2d002a8013002dull, 0x2e002a8018002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002a8008002bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64001c002e002eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2d002e8017002dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x640016002d002dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x640010002c002cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002c800a002bull, 0x29002c80010029ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002d800b002bull, 0x64000000290029ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2b002e800c002bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x640009002b002bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x640003002a002aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6400660035002full, 0x64006600360030ull, 0x64006600370031ull, 0x64006600380032ull, 0x64006600390033ull, 0x640066003a0034ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2f00230069002full, 0x30002400690030ull, 0x31002500690031ull, 0x32002600690032ull, 0x33002700690033ull, 0x34002800690034ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x2f0029006a002full, 0x30002a006a0030ull, 0x31002b006a0031ull, 0x32002c006a0032ull, 0x33002d006a0033ull, 0x34002e006a0034ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x30002f80020030ull, 0x31002f80070031ull, 0x32002f800d0032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x31003080080031ull, 0x320030800e0032ull, 0x33003080130033ull, 0x34003080180034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64001c00340034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x33003480170033ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64001600330033ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64001000320032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310032800a0031ull, 0x2f00328001002full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310033800b0031ull, 0x640000002f002full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x310034800c0031ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64000900310031ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
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
    0x64000300300030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
};
constexpr int TLM_OPS = 737;
static __device__ const double tlm_const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 2.0, 6.1697947043828245, -0.42772256543218573};
static __device__ const unsigned long long tlm_prog[737] = {
    0xaa00aa00aa008full, 0xaa00aa00aa0090ull, 0xaa00aa00aa0091ull, 0xaa00aa00aa0092ull, 0xaa00aa00aa0093ull, 0xaa00aa00aa0094ull, 0xaa00aa00aa00a1ull, 0xa900ab006f00a3ull,
    0xa100ab00a300a1ull, 0xa900a1004100a1ull, 0xa900ab001f00a2ull, 0xa100a2007300a1ull, 0x9100ab80a10091ull, 0x9000a100af0090ull, 0xaa00aa00aa00a1ull, 0xa9006e001f00a3ull,
    0xa100ab00a300a1ull, 0xa9006f001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1004200a1ull, 0xa9001f001e00a2ull, 0xa100a2007400a1ull, 0x9000ab80a10090ull, 0x9100ab80a10091ull,
    0x9200ab00a10092ull, 0xaa00aa00aa00a1ull, 0xa900ab007000a3ull, 0xa100ab00a300a1ull, 0xa900a1004300a1ull, 0xa900ab002000a2ull, 0xa100a2007500a1ull, 0x9200ab80a10092ull,
    0x9000ab00a10090ull, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa9006e002000a3ull, 0xa100ab00a300a1ull, 0xa90070001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1004400a1ull,
    0xa90020001e00a2ull, 0xa100a2007600a1ull, 0x9000ab80a10090ull, 0x9200ab80a10092ull, 0x9100a100af0091ull, 0xaa00aa00aa00a1ull, 0xa900ab007000a3ull, 0xa100ab00a300a1ull,
    0xa900a1004500a1ull, 0xa900ab002000a2ull, 0xa100a2007700a1ull, 0x9200ab80a10092ull, 0x8f00ab00a1008full, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa900ab006d00a3ull,
    0xa100ab00a300a1ull, 0xa900a1004600a1ull, 0xa900ab001d00a2ull, 0xa100a2007800a1ull, 0x8f00ab80a1008full, 0x9000ab00a10090ull, 0xaa00aa00aa00a1ull, 0xa9006d002000a3ull,
    0xa100ab00a300a1ull, 0xa90070001d00a3ull, 0xa100ab00a300a1ull, 0xa900a1004700a1ull, 0xa90020001d00a2ull, 0xa100a2007900a1ull, 0x8f00ab80a1008full, 0x9200ab80a10092ull,
    0x9100a100af0091ull, 0xaa00aa00aa00a1ull, 0xa90070002100a3ull, 0xa100ab00a300a1ull, 0xa90071002000a3ull, 0xa100ab00a300a1ull, 0xa900a1004800a1ull, 0xa90021002000a2ull,
    0xa100a2007a00a1ull, 0x9300ab80a10093ull, 0x9200ab80a10092ull, 0x9400ab00a10094ull, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa9006e002200a3ull, 0xa100ab00a300a1ull,
    0xa90072001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1004900a1ull, 0xa90022001e00a2ull, 0xa100a2007b00a1ull, 0x9400ab80a10094ull, 0x9000ab80a10090ull, 0x9300ab00a10093ull,
    0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa900ab007200a3ull, 0xa100ab00a300a1ull, 0xa900a1004a00a1ull, 0xa900ab002200a2ull, 0xa100a2007c00a1ull, 0x9400ab80a10094ull,
    0x9300ab00a10093ull, 0x9000ab00a10090ull, 0xa900ab008f007dull, 0xa900ab0090007eull, 0xa900ab0091007full, 0xa900ab00920080ull, 0xa900ab00930081ull, 0xa900ab00940082ull,
    0xaa00aa00aa00a1ull, 0xa900ab002500a3ull, 0xa100ab00a300a1ull, 0xa900a1007300a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004100a1ull, 0x7f00ab80a1007full, 0x7e00a100af007eull,
    0xaa00aa00aa00a1ull, 0xa90024001f00a3ull, 0xa100ab00a300a1ull, 0xa90025001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007400a1ull, 0xaa00aa00aa00a2ull, 0xa9006f002400a3ull,
    0xa200ab00a300a2ull, 0xa9006e002500a3ull, 0xa200ab00a300a2ull, 0xa100a2004200a1ull, 0x7e00ab80a1007eull, 0x7f00ab80a1007full, 0x8000ab00a10080ull, 0xaa00aa00aa00a1ull,
    0xa900ab002600a3ull, 0xa100ab00a300a1ull, 0xa900a1007500a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004300a1ull, 0x8000ab80a10080ull, 0x7e00ab00a1007eull, 0x7f00ab00a1007full,
    0xaa00aa00aa00a1ull, 0xa90024002000a3ull, 0xa100ab00a300a1ull, 0xa90026001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007600a1ull, 0xaa00aa00aa00a2ull, 0xa90070002400a3ull,
    0xa200ab00a300a2ull, 0xa9006e002600a3ull, 0xa200ab00a300a2ull, 0xa100a2004400a1ull, 0x7e00ab80a1007eull, 0x8000ab80a10080ull, 0x7f00a100af007full, 0xaa00aa00aa00a1ull,
    0xa900ab002600a3ull, 0xa100ab00a300a1ull, 0xa900a1007700a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004500a1ull, 0x8000ab80a10080ull, 0x7d00ab00a1007dull, 0x7f00ab00a1007full,
    0xaa00aa00aa00a1ull, 0xa900ab002300a3ull, 0xa100ab00a300a1ull, 0xa900a1007800a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004600a1ull, 0x7d00ab80a1007dull, 0x7e00ab00a1007eull,
    0xaa00aa00aa00a1ull, 0xa90023002000a3ull, 0xa100ab00a300a1ull, 0xa90026001d00a3ull, 0xa100ab00a300a1ull, 0xa900a1007900a1ull, 0xaa00aa00aa00a2ull, 0xa90070002300a3ull,
    0xa200ab00a300a2ull, 0xa9006d002600a3ull, 0xa200ab00a300a2ull, 0xa100a2004700a1ull, 0x7d00ab80a1007dull, 0x8000ab80a10080ull, 0x7f00a100af007full, 0xaa00aa00aa00a1ull,
    0xa90026002100a3ull, 0xa100ab00a300a1ull, 0xa90027002000a3ull, 0xa100ab00a300a1ull, 0xa900a1007a00a1ull, 0xaa00aa00aa00a2ull, 0xa90071002600a3ull, 0xa200ab00a300a2ull,
    0xa90070002700a3ull, 0xa200ab00a300a2ull, 0xa100a2004800a1ull, 0x8100ab80a10081ull, 0x8000ab80a10080ull, 0x8200ab00a10082ull, 0x7f00ab00a1007full, 0xaa00aa00aa00a1ull,
    0xa90024002200a3ull, 0xa100ab00a300a1ull, 0xa90028001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007b00a1ull, 0xaa00aa00aa00a2ull, 0xa90072002400a3ull, 0xa200ab00a300a2ull,
    0xa9006e002800a3ull, 0xa200ab00a300a2ull, 0xa100a2004900a1ull, 0x8200ab80a10082ull, 0x7e00ab80a1007eull, 0x8100ab00a10081ull, 0x7f00ab00a1007full, 0xaa00aa00aa00a1ull,
    0xa900ab002800a3ull, 0xa100ab00a300a1ull, 0xa900a1007c00a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004a00a1ull, 0x8200ab80a10082ull, 0x8100ab00a10081ull, 0x7e00ab00a1007eull,
    0x7e007d8002007eull, 0x7f007d8007007full, 0x7f007e8008007full, 0x80007d800d0080ull, 0x80007e800e0080ull, 0x80007f800f0080ull, 0x81007e80130081ull, 0x81007f80140081ull,
    0x81008080150081ull, 0x82007e80180082ull, 0x82007f80190082ull, 0x820080801a0082ull, 0x820081801b0082ull, 0xa9001c00820082ull, 0x81008280170081ull, 0xa9001600810081ull,
    0x80008180110080ull, 0x80008280120080ull, 0xa9001000800080ull, 0x7f0080800a007full, 0x7f0081800b007full, 0x7f0082800c007full, 0xa90009007f007full, 0x7e007f8004007eull,
    0x7e00808005007eull, 0x7e00828006007eull, 0xa90003007e007eull, 0x7d00808001007dull, 0xa90000007d007dull, 0xa900ab001d0095ull, 0xa900ab006d009bull, 0x9500ab00230095ull,
    0x9b00ab007d009bull, 0xa900ab001e0096ull, 0xa900ab006e009cull, 0x9600ab00240096ull, 0x9c00ab007e009cull, 0xa900ab001f0097ull, 0xa900ab006f009dull, 0x9700ab00250097ull,
    0x9d00ab007f009dull, 0xa900ab00200098ull, 0xa900ab0070009eull, 0x9800ab00260098ull, 0x9e00ab0080009eull, 0xa900ab00210099ull, 0xa900ab0071009full, 0x9900ab00270099ull,
    0x9f00ab0081009full, 0xa900ab0022009aull, 0xa900ab007200a0ull, 0x9a00ab0028009aull, 0xa000ab008200a0ull, 0xaa00aa00aa008full, 0xaa00aa00aa0090ull, 0xaa00aa00aa0091ull,
    0xaa00aa00aa0092ull, 0xaa00aa00aa0093ull, 0xaa00aa00aa0094ull, 0xaa00aa00aa00a1ull, 0xa900ab009d00a3ull, 0xa100ab00a300a1ull, 0xa900a1004100a1ull, 0xa900ab009700a2ull,
    0xa100a2007300a1ull, 0x9100ab80a10091ull, 0x9000a100af0090ull, 0xaa00aa00aa00a1ull, 0xa9009c009700a3ull, 0xa100ab00a300a1ull, 0xa9009d009600a3ull, 0xa100ab00a300a1ull,
    0xa900a1004200a1ull, 0xa90097009600a2ull, 0xa100a2007400a1ull, 0x9000ab80a10090ull, 0x9100ab80a10091ull, 0x9200ab00a10092ull, 0xaa00aa00aa00a1ull, 0xa900ab009e00a3ull,
    0xa100ab00a300a1ull, 0xa900a1004300a1ull, 0xa900ab009800a2ull, 0xa100a2007500a1ull, 0x9200ab80a10092ull, 0x9000ab00a10090ull, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull,
    0xa9009c009800a3ull, 0xa100ab00a300a1ull, 0xa9009e009600a3ull, 0xa100ab00a300a1ull, 0xa900a1004400a1ull, 0xa90098009600a2ull, 0xa100a2007600a1ull, 0x9000ab80a10090ull,
    0x9200ab80a10092ull, 0x9100a100af0091ull, 0xaa00aa00aa00a1ull, 0xa900ab009e00a3ull, 0xa100ab00a300a1ull, 0xa900a1004500a1ull, 0xa900ab009800a2ull, 0xa100a2007700a1ull,
    0x9200ab80a10092ull, 0x8f00ab00a1008full, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa900ab009b00a3ull, 0xa100ab00a300a1ull, 0xa900a1004600a1ull, 0xa900ab009500a2ull,
    0xa100a2007800a1ull, 0x8f00ab80a1008full, 0x9000ab00a10090ull, 0xaa00aa00aa00a1ull, 0xa9009b009800a3ull, 0xa100ab00a300a1ull, 0xa9009e009500a3ull, 0xa100ab00a300a1ull,
    0xa900a1004700a1ull, 0xa90098009500a2ull, 0xa100a2007900a1ull, 0x8f00ab80a1008full, 0x9200ab80a10092ull, 0x9100a100af0091ull, 0xaa00aa00aa00a1ull, 0xa9009e009900a3ull,
    0xa100ab00a300a1ull, 0xa9009f009800a3ull, 0xa100ab00a300a1ull, 0xa900a1004800a1ull, 0xa90099009800a2ull, 0xa100a2007a00a1ull, 0x9300ab80a10093ull, 0x9200ab80a10092ull,
    0x9400ab00a10094ull, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa9009c009a00a3ull, 0xa100ab00a300a1ull, 0xa900a0009600a3ull, 0xa100ab00a300a1ull, 0xa900a1004900a1ull,
    0xa9009a009600a2ull, 0xa100a2007b00a1ull, 0x9400ab80a10094ull, 0x9000ab80a10090ull, 0x9300ab00a10093ull, 0x9100ab00a10091ull, 0xaa00aa00aa00a1ull, 0xa900ab00a000a3ull,
    0xa100ab00a300a1ull, 0xa900a1004a00a1ull, 0xa900ab009a00a2ull, 0xa100a2007c00a1ull, 0x9400ab80a10094ull, 0x9300ab00a10093ull, 0x9000ab00a10090ull, 0xa900ab008f0083ull,
    0x83007d00ac0083ull, 0xa900ab00900084ull, 0x84007e00ac0084ull, 0xa900ab00910085ull, 0x85007f00ac0085ull, 0xa900ab00920086ull, 0x86008000ac0086ull, 0xa900ab00930087ull,
    0x87008100ac0087ull, 0xa900ab00940088ull, 0x88008200ac0088ull, 0xaa00aa00aa00a1ull, 0xa900ab002b00a3ull, 0xa100ab00a300a1ull, 0xa900a1007300a1ull, 0xaa00aa00aa00a2ull,
    0xa100a2004100a1ull, 0x8500ab80a10085ull, 0x8400a100af0084ull, 0xaa00aa00aa00a1ull, 0xa9002a001f00a3ull, 0xa100ab00a300a1ull, 0xa9002b001e00a3ull, 0xa100ab00a300a1ull,
    0xa900a1007400a1ull, 0xaa00aa00aa00a2ull, 0xa9006f002a00a3ull, 0xa200ab00a300a2ull, 0xa9006e002b00a3ull, 0xa200ab00a300a2ull, 0xa100a2004200a1ull, 0x8400ab80a10084ull,
    0x8500ab80a10085ull, 0x8600ab00a10086ull, 0xaa00aa00aa00a1ull, 0xa900ab002c00a3ull, 0xa100ab00a300a1ull, 0xa900a1007500a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004300a1ull,
    0x8600ab80a10086ull, 0x8400ab00a10084ull, 0x8500ab00a10085ull, 0xaa00aa00aa00a1ull, 0xa9002a002000a3ull, 0xa100ab00a300a1ull, 0xa9002c001e00a3ull, 0xa100ab00a300a1ull,
    0xa900a1007600a1ull, 0xaa00aa00aa00a2ull, 0xa90070002a00a3ull, 0xa200ab00a300a2ull, 0xa9006e002c00a3ull, 0xa200ab00a300a2ull, 0xa100a2004400a1ull, 0x8400ab80a10084ull,
    0x8600ab80a10086ull, 0x8500a100af0085ull, 0xaa00aa00aa00a1ull, 0xa900ab002c00a3ull, 0xa100ab00a300a1ull, 0xa900a1007700a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004500a1ull,
    0x8600ab80a10086ull, 0x8300ab00a10083ull, 0x8500ab00a10085ull, 0xaa00aa00aa00a1ull, 0xa900ab002900a3ull, 0xa100ab00a300a1ull, 0xa900a1007800a1ull, 0xaa00aa00aa00a2ull,
    0xa100a2004600a1ull, 0x8300ab80a10083ull, 0x8400ab00a10084ull, 0xaa00aa00aa00a1ull, 0xa90029002000a3ull, 0xa100ab00a300a1ull, 0xa9002c001d00a3ull, 0xa100ab00a300a1ull,
    0xa900a1007900a1ull, 0xaa00aa00aa00a2ull, 0xa90070002900a3ull, 0xa200ab00a300a2ull, 0xa9006d002c00a3ull, 0xa200ab00a300a2ull, 0xa100a2004700a1ull, 0x8300ab80a10083ull,
    0x8600ab80a10086ull, 0x8500a100af0085ull, 0xaa00aa00aa00a1ull, 0xa9002c002100a3ull, 0xa100ab00a300a1ull, 0xa9002d002000a3ull, 0xa100ab00a300a1ull, 0xa900a1007a00a1ull,
    0xaa00aa00aa00a2ull, 0xa90071002c00a3ull, 0xa200ab00a300a2ull, 0xa90070002d00a3ull, 0xa200ab00a300a2ull, 0xa100a2004800a1ull, 0x8700ab80a10087ull, 0x8600ab80a10086ull,
    0x8800ab00a10088ull, 0x8500ab00a10085ull, 0xaa00aa00aa00a1ull, 0xa9002a002200a3ull, 0xa100ab00a300a1ull, 0xa9002e001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007b00a1ull,
    0xaa00aa00aa00a2ull, 0xa90072002a00a3ull, 0xa200ab00a300a2ull, 0xa9006e002e00a3ull, 0xa200ab00a300a2ull, 0xa100a2004900a1ull, 0x8800ab80a10088ull, 0x8400ab80a10084ull,
    0x8700ab00a10087ull, 0x8500ab00a10085ull, 0xaa00aa00aa00a1ull, 0xa900ab002e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007c00a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004a00a1ull,
    0x8800ab80a10088ull, 0x8700ab00a10087ull, 0x8400ab00a10084ull, 0x84008380020084ull, 0x85008380070085ull, 0x85008480080085ull, 0x860083800d0086ull, 0x860084800e0086ull,
    0x860085800f0086ull, 0x87008480130087ull, 0x87008580140087ull, 0x87008680150087ull, 0x88008480180088ull, 0x88008580190088ull, 0x880086801a0088ull, 0x880087801b0088ull,
    0xa9001c00880088ull, 0x87008880170087ull, 0xa9001600870087ull, 0x86008780110086ull, 0x86008880120086ull, 0xa9001000860086ull, 0x850086800a0085ull, 0x850087800b0085ull,
    0x850088800c0085ull, 0xa9000900850085ull, 0x84008580040084ull, 0x84008680050084ull, 0x84008880060084ull, 0xa9000300840084ull, 0x83008680010083ull, 0xa9000000830083ull,
    0xa900ab008f0089ull, 0x89007d00ad0089ull, 0x89008300ae0089ull, 0xa900ab0090008aull, 0x8a007e00ad008aull, 0x8a008400ae008aull, 0xa900ab0091008bull, 0x8b007f00ad008bull,
    0x8b008500ae008bull, 0xa900ab0092008cull, 0x8c008000ad008cull, 0x8c008600ae008cull, 0xa900ab0093008dull, 0x8d008100ad008dull, 0x8d008700ae008dull, 0xa900ab0094008eull,
    0x8e008200ad008eull, 0x8e008800ae008eull, 0xaa00aa00aa00a1ull, 0xa900ab003100a3ull, 0xa100ab00a300a1ull, 0xa900a1007300a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004100a1ull,
    0x8b00ab80a1008bull, 0x8a00a100af008aull, 0xaa00aa00aa00a1ull, 0xa90030001f00a3ull, 0xa100ab00a300a1ull, 0xa90031001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007400a1ull,
    0xaa00aa00aa00a2ull, 0xa9006f003000a3ull, 0xa200ab00a300a2ull, 0xa9006e003100a3ull, 0xa200ab00a300a2ull, 0xa100a2004200a1ull, 0x8a00ab80a1008aull, 0x8b00ab80a1008bull,
    0x8c00ab00a1008cull, 0xaa00aa00aa00a1ull, 0xa900ab003200a3ull, 0xa100ab00a300a1ull, 0xa900a1007500a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004300a1ull, 0x8c00ab80a1008cull,
    0x8a00ab00a1008aull, 0x8b00ab00a1008bull, 0xaa00aa00aa00a1ull, 0xa90030002000a3ull, 0xa100ab00a300a1ull, 0xa90032001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007600a1ull,
    0xaa00aa00aa00a2ull, 0xa90070003000a3ull, 0xa200ab00a300a2ull, 0xa9006e003200a3ull, 0xa200ab00a300a2ull, 0xa100a2004400a1ull, 0x8a00ab80a1008aull, 0x8c00ab80a1008cull,
    0x8b00a100af008bull, 0xaa00aa00aa00a1ull, 0xa900ab003200a3ull, 0xa100ab00a300a1ull, 0xa900a1007700a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004500a1ull, 0x8c00ab80a1008cull,
    0x8900ab00a10089ull, 0x8b00ab00a1008bull, 0xaa00aa00aa00a1ull, 0xa900ab002f00a3ull, 0xa100ab00a300a1ull, 0xa900a1007800a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004600a1ull,
    0x8900ab80a10089ull, 0x8a00ab00a1008aull, 0xaa00aa00aa00a1ull, 0xa9002f002000a3ull, 0xa100ab00a300a1ull, 0xa90032001d00a3ull, 0xa100ab00a300a1ull, 0xa900a1007900a1ull,
    0xaa00aa00aa00a2ull, 0xa90070002f00a3ull, 0xa200ab00a300a2ull, 0xa9006d003200a3ull, 0xa200ab00a300a2ull, 0xa100a2004700a1ull, 0x8900ab80a10089ull, 0x8c00ab80a1008cull,
    0x8b00a100af008bull, 0xaa00aa00aa00a1ull, 0xa90032002100a3ull, 0xa100ab00a300a1ull, 0xa90033002000a3ull, 0xa100ab00a300a1ull, 0xa900a1007a00a1ull, 0xaa00aa00aa00a2ull,
    0xa90071003200a3ull, 0xa200ab00a300a2ull, 0xa90070003300a3ull, 0xa200ab00a300a2ull, 0xa100a2004800a1ull, 0x8d00ab80a1008dull, 0x8c00ab80a1008cull, 0x8e00ab00a1008eull,
    0x8b00ab00a1008bull, 0xaa00aa00aa00a1ull, 0xa90030002200a3ull, 0xa100ab00a300a1ull, 0xa90034001e00a3ull, 0xa100ab00a300a1ull, 0xa900a1007b00a1ull, 0xaa00aa00aa00a2ull,
    0xa90072003000a3ull, 0xa200ab00a300a2ull, 0xa9006e003400a3ull, 0xa200ab00a300a2ull, 0xa100a2004900a1ull, 0x8e00ab80a1008eull, 0x8a00ab80a1008aull, 0x8d00ab00a1008dull,
    0x8b00ab00a1008bull, 0xaa00aa00aa00a1ull, 0xa900ab003400a3ull, 0xa100ab00a300a1ull, 0xa900a1007c00a1ull, 0xaa00aa00aa00a2ull, 0xa100a2004a00a1ull, 0x8e00ab80a1008eull,
    0x8d00ab00a1008dull, 0x8a00ab00a1008aull, 0x8a00898002008aull, 0x8b00898007008bull, 0x8b008a8008008bull, 0x8c0089800d008cull, 0x8c008a800e008cull, 0x8c008b800f008cull,
    0x8d008a8013008dull, 0x8d008b8014008dull, 0x8d008c8015008dull, 0x8e008a8018008eull, 0x8e008b8019008eull, 0x8e008c801a008eull, 0x8e008d801b008eull, 0xa9001c008e008eull,
    0x8d008e8017008dull, 0xa90016008d008dull, 0x8c008d8011008cull, 0x8c008e8012008cull, 0xa90010008c008cull, 0x8b008c800a008bull, 0x8b008d800b008bull, 0x8b008e800c008bull,
    0xa90009008b008bull, 0x8a008b8004008aull, 0x8a008c8005008aull, 0x8a008e8006008aull, 0xa90003008a008aull, 0x89008c80010089ull, 0xa9000000890089ull, 0x6d00ab007d006dull,
    0x6d008300b0006dull, 0x6d008900b1006dull, 0x6e00ab007e006eull, 0x6e008400b0006eull, 0x6e008a00b1006eull, 0x6f00ab007f006full, 0x6f008500b0006full, 0x6f008b00b1006full,
    0x7000ab00800070ull, 0x70008600b00070ull, 0x70008c00b10070ull, 0x7100ab00810071ull, 0x71008700b00071ull, 0x71008d00b10071ull, 0x7200ab00820072ull, 0x72008800b00072ull,
    0x72008e00b10072ull,
};
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
  static constexpr int F = 53;
  static constexpr int DY = 59;
  static constexpr int KT = 65;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 75;
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

  // ---- warp-cooperative attempt (static warp schedules) ----
  static constexpr int NPART = 15;
  static constexpr int Q = 75;            // rates q_r, then q_i of the error norm
  static constexpr int D = 85;     // partial derivatives
  static constexpr int CB = 100;        // constants
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
      S[104] = -1.0156171083877703 / h;    // c21 / h
      S[105] = 4.0759956452537702 / h;    // c31 / h
      S[106] = 9.20767942983308 / h;    // c32 / h
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

  // ---- tangent of one accepted step (forward sensitivities) ----
  static constexpr int DYT = 109;     // dy in, dy_new out (NV)
  static constexpr int DKR = 115;     // dk, the rate constants' tangent (NR)
  static constexpr int TLM_CB = 169;  // constants of the tangent program
  static constexpr int TLM_NCONST = 9;
  static constexpr int NSLOTS_TLM = 178;
  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks
  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and
  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].
  template <class SA, class KA>
  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {
    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);
    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];
    S[172] = -1.0156171083877703 / h;    // c21 / h
    S[173] = 4.0759956452537702 / h;    // c31 / h
    S[174] = 9.20767942983308 / h;    // c32 / h
    for (int n = 0; n < coop::TLM_OPS; ++n) {
      const unsigned long long w = __ldg(coop::tlm_prog + n);
      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                            ((long long)(lo >> 31) << 63));
      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
    }
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
