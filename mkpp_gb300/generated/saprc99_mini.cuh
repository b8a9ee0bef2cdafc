// Generated by mkpp_gb300.emitter.cuda_emitter from mechanisms/saprc99_mini.plan.json.
// Do not edit: regenerate with `python -m mkpp_gb300.emitter.cuda_emitter`.
// 17 species (14 variable), 13 reactions, 46 W slots, 53 LU slots, 38 LU products, 24 pivot scalings.
#pragma once
#include "mkpp_device.cuh"
namespace mkpp_saprc99_mini {

// Tables of the warp-cooperative attempt (device constant data).
namespace coop {
static __device__ const double const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 0.0, -2.0, 2.0};
static __device__ const int stage_step[4] = {0, 41, 79, 111};
static __device__ const unsigned long long sched[3552] = {
    0xb800ba008900a4ull, 0xb80038008a00a5ull, 0xb8003f008a00a6ull, 0xb8003c008b00a7ull, 0xb8003f008b00a8ull, 0xb8003e008c00a9ull, 0xb8003c008c00aaull, 0xb80041008d00abull,
    0xb8003c008d00acull, 0xb80040008e00adull, 0xb8003e008e00aeull, 0xb80041008f00b0ull, 0xb8003d009100b2ull, 0xb8003b009100b3ull, 0xb800ba009200b4ull, 0xb800ba009300b5ull,
    0xb800ba009500b7ull, 0xb900b900b90019ull, 0xb900b900b9001full, 0xb900b900b90027ull, 0xb8004100890096ull, 0xb8003f008a0097ull, 0xb8003f008b0098ull, 0xb8003c008c0099ull,
    0xb8003c008d009aull, 0xb8003e008e009bull, 0xb80041008f009cull, 0xb8003b0091009eull, 0xb800390092009full, 0xb80037009300a0ull, 0xb8003d009400a1ull, 0xb8003a009500a2ull,
    0xbb00ba00b50002ull, 0xbb00ba00a60003ull, 0xb800bf00a80005ull, 0xb800ba00a50006ull, 0xbb00ba00b40007ull, 0xb800ba80b40008ull, 0xbb00ba00b70009ull, 0xb800ba80b5000aull,
    0xbb00ba00b2000cull, 0xb800ba80a6000eull, 0xbb00ba00a80010ull, 0xb800ba00aa0011ull, 0xb800ba80a50012ull, 0xb800ba00a90017ull, 0xbb00ba00aa0018ull, 0xb800ba00a6001cull,
    0xb800ba00a8001eull, 0xbb00ba00a50020ull, 0xb800ba80ab0024ull, 0xb800ba00ad0026ull, 0xbb00ba00ae0028ull, 0xb800ba80a9002bull, 0xb800ba80aa002dull, 0xb8003800970097ull,
    0xb8003c00980098ull, 0xb8003e00990099ull, 0xb80041009a009aull, 0xb80040009b009bull, 0xb80040009c009cull, 0xb8003d009e009eull, 0xb800ba009f0072ull, 0xb800ba80960079ull,
    0xb80040008f00afull, 0xb800ba009400b6ull, 0xb800ba80b40004ull, 0x600a700bf0006ull, 0xb800bf00b7000bull, 0xb800ba00b3000dull, 0x1000ba00a90010ull, 0x1200ba00a70012ull,
    0xb800ba00b20014ull, 0xbb00ba00b30015ull, 0x1800ba00ad0018ull, 0xb800ba00ae001aull, 0x2000ba00a70020ull, 0x2800ba00b00028ull, 0x2b00ba00ab002bull, 0x2d00ad00bf002dull,
    0xbb00ba00a40030ull, 0xb900b900b9002eull, 0x8000000000000002ull, 0x8000000000000003ull, 0x8000000000000007ull, 0xb800420090009dull, 0xb800ba80a0006full, 0xb800ba80970070ull,
    0xb800ba809f0071ull, 0x7200ba80a20072ull, 0xb800ba809e0073ull, 0xb800ba00970074ull, 0xb800ba00960076ull, 0xb800ba00960077ull, 0xb800ba009a0078ull, 0x7900ba00990079ull,
    0xd00ba80b6000dull, 0x1000ba00ab0010ull, 0xb800ba00ac0013ull, 0x1500ba00b60015ull, 0xb800ba80b50016ull, 0xb800ba80a4001bull, 0xb800ba80a40022ull, 0xb800ba80b20023ull,
    0xb800ba80b30025ull, 0xb800ba80ac0029ull, 0xb800bf00ae002full, 0x3000ba00ac0030ull, 0xb900b900b9000full, 0xb900b900b9001dull, 0xb900b900b90021ull, 0xb80002000a000aull,
    0xb80003000e000eull, 0xb80003001c001cull, 0xb8000700080008ull, 0x8000000000000009ull, 0x800000000000000cull, 0x70009800c00070ull, 0x7300ba00a00073ull, 0x7400ba80980074ull,
    0xb800ba809e0075ull, 0x7600ba80990076ull, 0x7700ba80970077ull, 0x7800ba809b0078ull, 0x7900ba809a0079ull, 0xb800ba006f0045ull, 0xb800ba00710047ull, 0xb800ba00720048ull,
    0xb800ba009000b1ull, 0xb800ba00bb0000ull, 0xb800ba00bb0001ull, 0x2900ba00af0029ull, 0xb800ba80b6002cull, 0x2f00ba00b0002full, 0x3000ba00af0030ull, 0xb800ba80b00032ull,
    0xb800ba80af0033ull, 0xb8000200160016ull, 0xf0004800e000full, 0x1d0004801c001dull, 0xb80009000b000bull, 0xb8000c00140014ull, 0xb8000c00230023ull, 0x100005800e0010ull,
    0x120006800e0012ull, 0x1e0005801c001eull, 0x200006801c0020ull, 0xb900b900b9006dull, 0xb900b900b9006eull, 0x7000ba009f0070ull, 0x7300ba00a10073ull, 0x7400ba80990074ull,
    0x7500ba80a10075ull, 0x7600ba809b0076ull, 0x7700ba80980077ull, 0x7800ba809c0078ull, 0x79009b00c00079ull, 0xb800ba009c007aull, 0x48004780080048ull, 0xffffull,
    0xb800ba80b1002aull, 0xb800ba80b10031ull, 0xbb00ba00b10034ull, 0x8000000000000000ull, 0x8000000000000001ull, 0xb80007000f000full, 0xb80007001d001dull, 0x8000000000000010ull,
    0x15000d80140015ull, 0x25000d80230025ull, 0x7300a200c00073ull, 0x7400ba809a0074ull, 0x7600ba00a00076ull, 0x7800ba009d0078ull, 0x7900ba809c0079ull, 0x7a00ba809d007aull,
    0xb800ba006d0043ull, 0xb800ba006e0044ull, 0xb800ba00700046ull, 0xb800ba0075004bull, 0xb800ba0077004dull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8001000170017ull, 0xb80010001e001eull, 0xb8001000240024ull, 0xb80010002b002bull, 0x8000000000000015ull, 0x7800ba009e0078ull, 0x7900ba009d0079ull, 0xb800ba00730049ull,
    0xb800ba0074004aull, 0xb800ba0076004cull, 0xb800ba007a0050ull, 0x4d0046801c004dull, 0xb8000100440044ull, 0xb8000000430043ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8001500250025ull, 0xb80015002c002cull, 0x18001180170018ull, 0x19001280170019ull, 0x1b00138017001bull, 0x1f0011801e001full, 0x26001180240026ull, 0x2d0011802b002dull,
    0x200012801e0020ull, 0x220013801e0022ull, 0x27001280240027ull, 0x2e0012802b002eull, 0x29001380240029ull, 0x300013802b0030ull, 0x7900ba00a10079ull, 0xb800ba0078004eull,
    0x490045800a0049ull, 0x4a0046800e004aull, 0x4c00458016004cull, 0x4d0047801d004dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000018ull, 0xb800ba0079004full, 0x490048800b0049ull, 0x4a0047800f004aull, 0xb8000200450045ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80018001f001full, 0xb8001800260026ull, 0xb80018002d002dull, 0x4b00498014004bull, 0x4c004a8017004cull, 0x4d004a801e004dull, 0x4e00498023004eull, 0x4f004a802b004full,
    0xb8000900480048ull, 0xb8000700470047ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x200019801f0020ull, 0x21001a801f0021ull, 0x22001b801f0022ull, 0x27001980260027ull, 0x2e0019802d002eull, 0x28001a80260028ull, 0x29001b80260029ull, 0x2f001a802d002full,
    0x30001b802d0030ull, 0x4d004c801f004dull, 0x4e004a8024004eull, 0x4f004b802c004full, 0x46004780040046ull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000020ull, 0x4e004b8025004eull, 0x4f004c802d004full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8002000270027ull, 0xb80020002e002eull, 0x4e004c8026004eull, 0xb80015004b004bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x28002180270028ull, 0x29002280270029ull, 0x2f0021802e002full, 0x300022802e0030ull, 0x4e004d8027004eull, 0x4f004d802e004full, 0x49004b800d0049ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000028ull, 0xb8000c00490049ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80028002f002full, 0xb8002800320032ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x300029802f0030ull, 0x31002a802f0031ull, 0x33002980320033ull, 0x34002a80320034ull, 0x4f004e802f004full, 0x50004e80320050ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000030ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8003000330033ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x34003180330034ull, 0x50004f80330050ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x8000000000000034ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8003400500050ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4f00508031004full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80030004f004full, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4e004f8029004eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4e0050802a004eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80028004e004eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4d004e8021004dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4d004f8022004dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80020004d004dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4c004d8019004cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4c004e801a004cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4c004f801b004cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80018004c004cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4a004c8011004aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4a004d8012004aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x4a004f8013004aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80010004a004aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x46004a80050046ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x46004d80060046ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8000300460046ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x3500ba0043007bull, 0x3600ba0044007cull, 0x3700ba0045007dull, 0x3800ba0046007eull, 0x3900ba0047007full, 0x3a00ba00480080ull, 0x3b00ba00490081ull, 0x3c00ba004a0082ull,
    0x3d00ba004b0083ull, 0x3e00ba004c0084ull, 0x3f00ba004d0085ull, 0x4000ba004e0086ull, 0x4100ba004f0087ull, 0x4200ba00500088ull, 0xb900b900b9006dull, 0xb900b900b9006eull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8008700890096ull, 0xb80085008a0097ull, 0xb80085008b0098ull, 0xb80082008c0099ull, 0xb80082008d009aull, 0xb80084008e009bull, 0xb80087008f009cull, 0xb800880090009dull,
    0xb800810091009eull, 0xb8007f0092009full, 0xb8007d009300a0ull, 0xb80083009400a1ull, 0xb80080009500a2ull, 0xb800ba006d0051ull, 0xb800ba006e0052ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8007e00970097ull, 0xb8008200980098ull, 0xb8008400990099ull, 0xb80087009a009aull, 0xb80086009b009bull, 0xb80086009c009cull, 0xb80083009e009eull, 0xb800ba80a0006full,
    0xb800ba809f0071ull, 0xb800ba009f0072ull, 0xb800ba00960076ull, 0xb800ba00960077ull, 0xb800ba80960079ull, 0x51004300bc0051ull, 0x52004400bc0052ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb800ba80970070ull, 0x7200ba80a20072ull, 0xb800ba809e0073ull, 0xb800ba00970074ull, 0xb800ba809e0075ull, 0x7600ba80990076ull, 0x7700ba80970077ull, 0xb800ba009a0078ull,
    0x7900ba00990079ull, 0xb800ba009c007aull, 0xb800ba006f0053ull, 0xb800ba00710055ull, 0xb8000100520052ull, 0xb8000000510051ull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x70009800c00070ull, 0x7300ba00a00073ull, 0x7400ba80980074ull, 0x7500ba80a10075ull, 0x7600ba809b0076ull, 0x7700ba80980077ull, 0x7800ba809b0078ull, 0x7900ba809a0079ull,
    0x7a00ba809d007aull, 0x53004500bc0053ull, 0x55004700bc0055ull, 0xb800ba00720056ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x7000ba009f0070ull, 0x7300ba00a10073ull, 0x7400ba80990074ull, 0x7600ba00a00076ull, 0x7800ba809c0078ull, 0x79009b00c00079ull, 0x56004800bc0056ull, 0xb800ba00750059ull,
    0xb800ba0077005bull, 0xb800ba007a005eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x7300a200c00073ull, 0x7400ba809a0074ull, 0x7800ba009d0078ull, 0x7900ba809c0079ull, 0xb800ba00700054ull, 0x59004b00bc0059ull, 0xb800ba0076005aull, 0x5b004d00bc005bull,
    0x5e005000bc005eull, 0x56005580080056ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x7800ba009e0078ull, 0x7900ba009d0079ull, 0x54004600bc0054ull, 0xb800ba00730057ull, 0xb800ba00740058ull, 0x5a004c00bc005aull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x7900ba00a10079ull, 0x57004900bc0057ull, 0x58004a00bc0058ull, 0xb800ba0078005cull, 0x5a00538016005aull, 0x5b0054801c005bull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c004e00bc005cull, 0xb800ba0079005dull, 0x570053800a0057ull, 0x580054800e0058ull, 0x5b0055801d005bull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5d004f00bc005dull, 0x570056800b0057ull, 0x580055800f0058ull, 0xb8000200530053ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x59005780140059ull, 0x5a00588017005aull, 0x5b0058801e005bull, 0x5c00578023005cull, 0x5d0058802b005dull, 0xb8000900560056ull, 0xb8000700550055ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5b005a801f005bull, 0x5c00588024005cull, 0x5d0059802c005dull, 0x54005580040054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c00598025005cull, 0x5d005a802d005dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c005a8026005cull, 0x5d005b802e005dull, 0xb8001500590059ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c005b8027005cull, 0x570059800d0057ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5d005c802f005dull, 0x5e005c8032005eull, 0xb8000c00570057ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5e005d8033005eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80034005e005eull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5d005e8031005dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80030005d005dull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c005d8029005cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5c005e802a005cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80028005c005cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5b005c8021005bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5b005d8022005bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80020005b005bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5a005b8019005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5a005c801a005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5a005d801b005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80018005a005aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x58005a80110058ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x58005b80120058ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x58005d80130058ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8001000580058ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x54005880050054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x54005b80060054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8000300540054ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb800ba006d005full, 0xb800ba006e0060ull, 0xb800ba006f0061ull, 0xb800ba00700062ull, 0xb800ba00710063ull, 0xb800ba00720064ull, 0xb800ba00730065ull, 0xb800ba00740066ull,
    0xb800ba00750067ull, 0xb800ba00760068ull, 0xb800ba00770069ull, 0xb800ba0078006aull, 0xb800ba0079006bull, 0xb800ba007a006cull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5f004300bd005full, 0x60004400bd0060ull, 0x61004500bd0061ull, 0x62004600bd0062ull, 0x63004700bd0063ull, 0x64004800bd0064ull, 0x65004900bd0065ull, 0x66004a00bd0066ull,
    0x67004b00bd0067ull, 0x68004c00bd0068ull, 0x69004d00bd0069ull, 0x6a004e00bd006aull, 0x6b004f00bd006bull, 0x6c005000bd006cull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x5f005100be005full, 0x60005200be0060ull, 0x61005300be0061ull, 0x62005400be0062ull, 0x63005500be0063ull, 0x64005600be0064ull, 0x65005700be0065ull, 0x66005800be0066ull,
    0x67005900be0067ull, 0x68005a00be0068ull, 0x69005b00be0069ull, 0x6a005c00be006aull, 0x6b005d00be006bull, 0x6c005e00be006cull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x64006380080064ull, 0x650061800a0065ull, 0x660062800e0066ull, 0x68006180160068ull, 0x690062801c0069ull, 0xb8000100600060ull, 0xb80000005f005full, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x650064800b0065ull, 0x660063800f0066ull, 0x690063801d0069ull, 0xb8000200610061ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x67006580140067ull, 0x68006680170068ull, 0x690066801e0069ull, 0x6a00658023006aull, 0x6b0066802b006bull, 0xb8000900640064ull, 0xb8000700630063ull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x690068801f0069ull, 0x6a00668024006aull, 0x6b0067802c006bull, 0x62006380040062ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a00678025006aull, 0x6b0068802d006bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a00688026006aull, 0x6b0069802e006bull, 0xb8001500670067ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a00698027006aull, 0x650067800d0065ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6b006a802f006bull, 0x6c006a8032006cull, 0xb8000c00650065ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6c006b8033006cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80034006c006cull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6b006c8031006bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80030006b006bull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a006b8029006aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x6a006c802a006aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb80028006a006aull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x69006a80210069ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x69006b80220069ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8002000690069ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x68006980190068ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x68006a801a0068ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x68006b801b0068ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8001800680068ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x66006880110066ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x66006980120066ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x66006b80130066ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8001000660066ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x62006680050062ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0x62006980060062ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xb8000300620062ull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
    0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull, 0xffffull,
};
constexpr int TLM_OPS = 1103;
static __device__ const double tlm_const_val[9] = {-0.0, 0.0, 1.0, 0.0, 0.0, 0.0, 2.0, 6.1697947043828245, -0.42772256543218573};
static __device__ const unsigned long long tlm_prog[1103] = {
    0x139013901390106ull, 0x139013901390107ull, 0x139013901390108ull, 0x139013901390109ull, 0x13901390139010aull, 0x13901390139010bull, 0x13901390139010cull, 0x13901390139010dull,
    0x13901390139010eull, 0x13901390139010full, 0x139013901390110ull, 0x139013901390111ull, 0x139013901390112ull, 0x139013901390113ull, 0x139013901390130ull, 0x138013a00cd0132ull,
    0x130013a01320130ull, 0x138013000890130ull, 0x138013a00410131ull, 0x130013100cf0130ull, 0x112013a81300112ull, 0x10f013a0130010full, 0x110013a01300110ull, 0x139013901390130ull,
    0x13800c4003f0132ull, 0x130013a01320130ull, 0x13800cb00380132ull, 0x130013a01320130ull, 0x1380130008a0130ull, 0x138003f00380131ull, 0x130013100d00130ull, 0x110013a81300110ull,
    0x109013a81300109ull, 0x10d013a0130010dull, 0x139013901390130ull, 0x13800c8003f0132ull, 0x130013a01320130ull, 0x13800cb003c0132ull, 0x130013a01320130ull, 0x1380130008b0130ull,
    0x138003f003c0131ull, 0x130013100d10130ull, 0x110013a81300110ull, 0x10d013a8130010dull, 0x1090130013e0109ull, 0x139013901390130ull, 0x13800c8003e0132ull, 0x130013a01320130ull,
    0x13800ca003c0132ull, 0x130013a01320130ull, 0x1380130008c0130ull, 0x138003e003c0131ull, 0x130013100d20130ull, 0x10d013a8130010dull, 0x10f013a8130010full, 0x112013a01300112ull,
    0x139013901390130ull, 0x13800c800410132ull, 0x130013a01320130ull, 0x13800cd003c0132ull, 0x130013a01320130ull, 0x1380130008d0130ull, 0x1380041003c0131ull, 0x130013100d30130ull,
    0x10d013a8130010dull, 0x112013a81300112ull, 0x111013a01300111ull, 0x139013901390130ull, 0x13800ca00400132ull, 0x130013a01320130ull, 0x13800cc003e0132ull, 0x130013a01320130ull,
    0x1380130008e0130ull, 0x1380040003e0131ull, 0x130013100d40130ull, 0x10f013a8130010full, 0x111013a81300111ull, 0x1120130013e0112ull, 0x139013901390130ull, 0x13800cc00410132ull,
    0x130013a01320130ull, 0x13800cd00400132ull, 0x130013a01320130ull, 0x1380130008f0130ull, 0x138004100400131ull, 0x130013100d50130ull, 0x112013a81300112ull, 0x111013a81300111ull,
    0x113013a01300113ull, 0x139013901390130ull, 0x138013a00ce0132ull, 0x130013a01320130ull, 0x138013000900130ull, 0x138013a00420131ull, 0x130013100d60130ull, 0x113013a81300113ull,
    0x112013a01300112ull, 0x111013a01300111ull, 0x139013901390130ull, 0x13800c7003d0132ull, 0x130013a01320130ull, 0x13800c9003b0132ull, 0x130013a01320130ull, 0x138013000910130ull,
    0x138003d003b0131ull, 0x130013100d70130ull, 0x10c013a8130010cull, 0x10e013a8130010eull, 0x111013a01300111ull, 0x139013901390130ull, 0x138013a00c50132ull, 0x130013a01320130ull,
    0x138013000920130ull, 0x138013a00390131ull, 0x130013100d80130ull, 0x10a013a8130010aull, 0x10b013a0130010bull, 0x109013a01300109ull, 0x139013901390130ull, 0x138013a00c30132ull,
    0x130013a01320130ull, 0x138013000930130ull, 0x138013a00370131ull, 0x130013100d90130ull, 0x108013a81300108ull, 0x10c013a0130010cull, 0x10f013a0130010full, 0x139013901390130ull,
    0x138013a00c90132ull, 0x130013a01320130ull, 0x138013000940130ull, 0x138013a003d0131ull, 0x130013100da0130ull, 0x10e013a8130010eull, 0x10c013a0130010cull, 0x112013a01300112ull,
    0x139013901390130ull, 0x138013a00c60132ull, 0x130013a01320130ull, 0x138013000950130ull, 0x138013a003a0131ull, 0x130013100db0130ull, 0x10b013a8130010bull, 0x10c0130013e010cull,
    0x138013a010600dcull, 0x138013a010700ddull, 0x138013a010800deull, 0x138013a010900dfull, 0x138013a010a00e0ull, 0x138013a010b00e1ull, 0x138013a010c00e2ull, 0x138013a010d00e3ull,
    0x138013a010e00e4ull, 0x138013a010f00e5ull, 0x138013a011000e6ull, 0x138013a011100e7ull, 0x138013a011200e8ull, 0x138013a011300e9ull, 0x139013901390130ull, 0x138013a004f0132ull,
    0x130013a01320130ull, 0x138013000cf0130ull, 0x139013901390131ull, 0x130013100890130ull, 0xe8013a813000e8ull, 0xe5013a013000e5ull, 0xe6013a013000e6ull, 0x139013901390130ull,
    0x1380046003f0132ull, 0x130013a01320130ull, 0x138004d00380132ull, 0x130013a01320130ull, 0x138013000d00130ull, 0x139013901390131ull, 0x13800cb00460132ull, 0x131013a01320131ull,
    0x13800c4004d0132ull, 0x131013a01320131ull, 0x1300131008a0130ull, 0xe6013a813000e6ull, 0xdf013a813000dfull, 0xe3013a013000e3ull, 0x139013901390130ull, 0x138004a003f0132ull,
    0x130013a01320130ull, 0x138004d003c0132ull, 0x130013a01320130ull, 0x138013000d10130ull, 0x139013901390131ull, 0x13800cb004a0132ull, 0x131013a01320131ull, 0x13800c8004d0132ull,
    0x131013a01320131ull, 0x1300131008b0130ull, 0xe6013a813000e6ull, 0xe3013a813000e3ull, 0xdf0130013e00dfull, 0x139013901390130ull, 0x138004a003e0132ull, 0x130013a01320130ull,
    0x138004c003c0132ull, 0x130013a01320130ull, 0x138013000d20130ull, 0x139013901390131ull, 0x13800ca004a0132ull, 0x131013a01320131ull, 0x13800c8004c0132ull, 0x131013a01320131ull,
    0x1300131008c0130ull, 0xe3013a813000e3ull, 0xe5013a813000e5ull, 0xe8013a013000e8ull, 0x139013901390130ull, 0x138004a00410132ull, 0x130013a01320130ull, 0x138004f003c0132ull,
    0x130013a01320130ull, 0x138013000d30130ull, 0x139013901390131ull, 0x13800cd004a0132ull, 0x131013a01320131ull, 0x13800c8004f0132ull, 0x131013a01320131ull, 0x1300131008d0130ull,
    0xe3013a813000e3ull, 0xe8013a813000e8ull, 0xe7013a013000e7ull, 0x139013901390130ull, 0x138004c00400132ull, 0x130013a01320130ull, 0x138004e003e0132ull, 0x130013a01320130ull,
    0x138013000d40130ull, 0x139013901390131ull, 0x13800cc004c0132ull, 0x131013a01320131ull, 0x13800ca004e0132ull, 0x131013a01320131ull, 0x1300131008e0130ull, 0xe5013a813000e5ull,
    0xe7013a813000e7ull, 0xe80130013e00e8ull, 0x139013901390130ull, 0x138004e00410132ull, 0x130013a01320130ull, 0x138004f00400132ull, 0x130013a01320130ull, 0x138013000d50130ull,
    0x139013901390131ull, 0x13800cd004e0132ull, 0x131013a01320131ull, 0x13800cc004f0132ull, 0x131013a01320131ull, 0x1300131008f0130ull, 0xe8013a813000e8ull, 0xe7013a813000e7ull,
    0xe9013a013000e9ull, 0x139013901390130ull, 0x138013a00500132ull, 0x130013a01320130ull, 0x138013000d60130ull, 0x139013901390131ull, 0x130013100900130ull, 0xe9013a813000e9ull,
    0xe8013a013000e8ull, 0xe7013a013000e7ull, 0x139013901390130ull, 0x1380049003d0132ull, 0x130013a01320130ull, 0x138004b003b0132ull, 0x130013a01320130ull, 0x138013000d70130ull,
    0x139013901390131ull, 0x13800c900490132ull, 0x131013a01320131ull, 0x13800c7004b0132ull, 0x131013a01320131ull, 0x130013100910130ull, 0xe2013a813000e2ull, 0xe4013a813000e4ull,
    0xe7013a013000e7ull, 0x139013901390130ull, 0x138013a00470132ull, 0x130013a01320130ull, 0x138013000d80130ull, 0x139013901390131ull, 0x130013100920130ull, 0xe0013a813000e0ull,
    0xe1013a013000e1ull, 0xdf013a013000dfull, 0x139013901390130ull, 0x138013a00450132ull, 0x130013a01320130ull, 0x138013000d90130ull, 0x139013901390131ull, 0x130013100930130ull,
    0xde013a813000deull, 0xe2013a013000e2ull, 0xe5013a013000e5ull, 0x139013901390130ull, 0x138013a004b0132ull, 0x130013a01320130ull, 0x138013000da0130ull, 0x139013901390131ull,
    0x130013100940130ull, 0xe4013a813000e4ull, 0xe2013a013000e2ull, 0xe8013a013000e8ull, 0x139013901390130ull, 0x138013a00480132ull, 0x130013a01320130ull, 0x138013000db0130ull,
    0x139013901390131ull, 0x130013100950130ull, 0xe1013a813000e1ull, 0xe20130013e00e2ull, 0xe100e0800800e1ull, 0xe200de800a00e2ull, 0xe200e1800b00e2ull, 0xe300df800e00e3ull,
    0xe300e0800f00e3ull, 0xe400e2801400e4ull, 0xe500de801600e5ull, 0xe500e3801700e5ull, 0xe600df801c00e6ull, 0xe600e0801d00e6ull, 0xe600e3801e00e6ull, 0xe600e5801f00e6ull,
    0xe700e2802300e7ull, 0xe700e3802400e7ull, 0xe700e4802500e7ull, 0xe700e5802600e7ull, 0xe700e6802700e7ull, 0xe800e3802b00e8ull, 0xe800e4802c00e8ull, 0xe800e5802d00e8ull,
    0xe800e6802e00e8ull, 0xe800e7802f00e8ull, 0xe900e7803200e9ull, 0xe900e8803300e9ull, 0x138003400e900e9ull, 0xe800e9803100e8ull, 0x138003000e800e8ull, 0xe700e8802900e7ull,
    0xe700e9802a00e7ull, 0x138002800e700e7ull, 0xe600e7802100e6ull, 0xe600e8802200e6ull, 0x138002000e600e6ull, 0xe500e6801900e5ull, 0xe500e7801a00e5ull, 0xe500e8801b00e5ull,
    0x138001800e500e5ull, 0x138001500e400e4ull, 0xe300e5801100e3ull, 0xe300e6801200e3ull, 0xe300e8801300e3ull, 0x138001000e300e3ull, 0xe200e4800d00e2ull, 0x138000c00e200e2ull,
    0x138000900e100e1ull, 0x138000700e000e0ull, 0xdf00e0800400dfull, 0xdf00e3800500dfull, 0xdf00e6800600dfull, 0x138000300df00dfull, 0x138000200de00deull, 0x138000100dd00ddull,
    0x138000000dc00dcull, 0x138013a00350114ull, 0x138013a00c10122ull, 0x114013a00430114ull, 0x122013a00dc0122ull, 0x138013a00360115ull, 0x138013a00c20123ull, 0x115013a00440115ull,
    0x123013a00dd0123ull, 0x138013a00370116ull, 0x138013a00c30124ull, 0x116013a00450116ull, 0x124013a00de0124ull, 0x138013a00380117ull, 0x138013a00c40125ull, 0x117013a00460117ull,
    0x125013a00df0125ull, 0x138013a00390118ull, 0x138013a00c50126ull, 0x118013a00470118ull, 0x126013a00e00126ull, 0x138013a003a0119ull, 0x138013a00c60127ull, 0x119013a00480119ull,
    0x127013a00e10127ull, 0x138013a003b011aull, 0x138013a00c70128ull, 0x11a013a0049011aull, 0x128013a00e20128ull, 0x138013a003c011bull, 0x138013a00c80129ull, 0x11b013a004a011bull,
    0x129013a00e30129ull, 0x138013a003d011cull, 0x138013a00c9012aull, 0x11c013a004b011cull, 0x12a013a00e4012aull, 0x138013a003e011dull, 0x138013a00ca012bull, 0x11d013a004c011dull,
    0x12b013a00e5012bull, 0x138013a003f011eull, 0x138013a00cb012cull, 0x11e013a004d011eull, 0x12c013a00e6012cull, 0x138013a0040011full, 0x138013a00cc012dull, 0x11f013a004e011full,
    0x12d013a00e7012dull, 0x138013a00410120ull, 0x138013a00cd012eull, 0x120013a004f0120ull, 0x12e013a00e8012eull, 0x138013a00420121ull, 0x138013a00ce012full, 0x121013a00500121ull,
    0x12f013a00e9012full, 0x139013901390106ull, 0x139013901390107ull, 0x139013901390108ull, 0x139013901390109ull, 0x13901390139010aull, 0x13901390139010bull, 0x13901390139010cull,
    0x13901390139010dull, 0x13901390139010eull, 0x13901390139010full, 0x139013901390110ull, 0x139013901390111ull, 0x139013901390112ull, 0x139013901390113ull, 0x139013901390130ull,
    0x138013a012e0132ull, 0x130013a01320130ull, 0x138013000890130ull, 0x138013a01200131ull, 0x130013100cf0130ull, 0x112013a81300112ull, 0x10f013a0130010full, 0x110013a01300110ull,
    0x139013901390130ull, 0x1380125011e0132ull, 0x130013a01320130ull, 0x138012c01170132ull, 0x130013a01320130ull, 0x1380130008a0130ull, 0x138011e01170131ull, 0x130013100d00130ull,
    0x110013a81300110ull, 0x109013a81300109ull, 0x10d013a0130010dull, 0x139013901390130ull, 0x1380129011e0132ull, 0x130013a01320130ull, 0x138012c011b0132ull, 0x130013a01320130ull,
    0x1380130008b0130ull, 0x138011e011b0131ull, 0x130013100d10130ull, 0x110013a81300110ull, 0x10d013a8130010dull, 0x1090130013e0109ull, 0x139013901390130ull, 0x1380129011d0132ull,
    0x130013a01320130ull, 0x138012b011b0132ull, 0x130013a01320130ull, 0x1380130008c0130ull, 0x138011d011b0131ull, 0x130013100d20130ull, 0x10d013a8130010dull, 0x10f013a8130010full,
    0x112013a01300112ull, 0x139013901390130ull, 0x138012901200132ull, 0x130013a01320130ull, 0x138012e011b0132ull, 0x130013a01320130ull, 0x1380130008d0130ull, 0x1380120011b0131ull,
    0x130013100d30130ull, 0x10d013a8130010dull, 0x112013a81300112ull, 0x111013a01300111ull, 0x139013901390130ull, 0x138012b011f0132ull, 0x130013a01320130ull, 0x138012d011d0132ull,
    0x130013a01320130ull, 0x1380130008e0130ull, 0x138011f011d0131ull, 0x130013100d40130ull, 0x10f013a8130010full, 0x111013a81300111ull, 0x1120130013e0112ull, 0x139013901390130ull,
    0x138012d01200132ull, 0x130013a01320130ull, 0x138012e011f0132ull, 0x130013a01320130ull, 0x1380130008f0130ull, 0x1380120011f0131ull, 0x130013100d50130ull, 0x112013a81300112ull,
    0x111013a81300111ull, 0x113013a01300113ull, 0x139013901390130ull, 0x138013a012f0132ull, 0x130013a01320130ull, 0x138013000900130ull, 0x138013a01210131ull, 0x130013100d60130ull,
    0x113013a81300113ull, 0x112013a01300112ull, 0x111013a01300111ull, 0x139013901390130ull, 0x1380128011c0132ull, 0x130013a01320130ull, 0x138012a011a0132ull, 0x130013a01320130ull,
    0x138013000910130ull, 0x138011c011a0131ull, 0x130013100d70130ull, 0x10c013a8130010cull, 0x10e013a8130010eull, 0x111013a01300111ull, 0x139013901390130ull, 0x138013a01260132ull,
    0x130013a01320130ull, 0x138013000920130ull, 0x138013a01180131ull, 0x130013100d80130ull, 0x10a013a8130010aull, 0x10b013a0130010bull, 0x109013a01300109ull, 0x139013901390130ull,
    0x138013a01240132ull, 0x130013a01320130ull, 0x138013000930130ull, 0x138013a01160131ull, 0x130013100d90130ull, 0x108013a81300108ull, 0x10c013a0130010cull, 0x10f013a0130010full,
    0x139013901390130ull, 0x138013a012a0132ull, 0x130013a01320130ull, 0x138013000940130ull, 0x138013a011c0131ull, 0x130013100da0130ull, 0x10e013a8130010eull, 0x10c013a0130010cull,
    0x112013a01300112ull, 0x139013901390130ull, 0x138013a01270132ull, 0x130013a01320130ull, 0x138013000950130ull, 0x138013a01190131ull, 0x130013100db0130ull, 0x10b013a8130010bull,
    0x10c0130013e010cull, 0x138013a010600eaull, 0xea00dc013b00eaull, 0x138013a010700ebull, 0xeb00dd013b00ebull, 0x138013a010800ecull, 0xec00de013b00ecull, 0x138013a010900edull,
    0xed00df013b00edull, 0x138013a010a00eeull, 0xee00e0013b00eeull, 0x138013a010b00efull, 0xef00e1013b00efull, 0x138013a010c00f0ull, 0xf000e2013b00f0ull, 0x138013a010d00f1ull,
    0xf100e3013b00f1ull, 0x138013a010e00f2ull, 0xf200e4013b00f2ull, 0x138013a010f00f3ull, 0xf300e5013b00f3ull, 0x138013a011000f4ull, 0xf400e6013b00f4ull, 0x138013a011100f5ull,
    0xf500e7013b00f5ull, 0x138013a011200f6ull, 0xf600e8013b00f6ull, 0x138013a011300f7ull, 0xf700e9013b00f7ull, 0x139013901390130ull, 0x138013a005d0132ull, 0x130013a01320130ull,
    0x138013000cf0130ull, 0x139013901390131ull, 0x130013100890130ull, 0xf6013a813000f6ull, 0xf3013a013000f3ull, 0xf4013a013000f4ull, 0x139013901390130ull, 0x1380054003f0132ull,
    0x130013a01320130ull, 0x138005b00380132ull, 0x130013a01320130ull, 0x138013000d00130ull, 0x139013901390131ull, 0x13800cb00540132ull, 0x131013a01320131ull, 0x13800c4005b0132ull,
    0x131013a01320131ull, 0x1300131008a0130ull, 0xf4013a813000f4ull, 0xed013a813000edull, 0xf1013a013000f1ull, 0x139013901390130ull, 0x1380058003f0132ull, 0x130013a01320130ull,
    0x138005b003c0132ull, 0x130013a01320130ull, 0x138013000d10130ull, 0x139013901390131ull, 0x13800cb00580132ull, 0x131013a01320131ull, 0x13800c8005b0132ull, 0x131013a01320131ull,
    0x1300131008b0130ull, 0xf4013a813000f4ull, 0xf1013a813000f1ull, 0xed0130013e00edull, 0x139013901390130ull, 0x1380058003e0132ull, 0x130013a01320130ull, 0x138005a003c0132ull,
    0x130013a01320130ull, 0x138013000d20130ull, 0x139013901390131ull, 0x13800ca00580132ull, 0x131013a01320131ull, 0x13800c8005a0132ull, 0x131013a01320131ull, 0x1300131008c0130ull,
    0xf1013a813000f1ull, 0xf3013a813000f3ull, 0xf6013a013000f6ull, 0x139013901390130ull, 0x138005800410132ull, 0x130013a01320130ull, 0x138005d003c0132ull, 0x130013a01320130ull,
    0x138013000d30130ull, 0x139013901390131ull, 0x13800cd00580132ull, 0x131013a01320131ull, 0x13800c8005d0132ull, 0x131013a01320131ull, 0x1300131008d0130ull, 0xf1013a813000f1ull,
    0xf6013a813000f6ull, 0xf5013a013000f5ull, 0x139013901390130ull, 0x138005a00400132ull, 0x130013a01320130ull, 0x138005c003e0132ull, 0x130013a01320130ull, 0x138013000d40130ull,
    0x139013901390131ull, 0x13800cc005a0132ull, 0x131013a01320131ull, 0x13800ca005c0132ull, 0x131013a01320131ull, 0x1300131008e0130ull, 0xf3013a813000f3ull, 0xf5013a813000f5ull,
    0xf60130013e00f6ull, 0x139013901390130ull, 0x138005c00410132ull, 0x130013a01320130ull, 0x138005d00400132ull, 0x130013a01320130ull, 0x138013000d50130ull, 0x139013901390131ull,
    0x13800cd005c0132ull, 0x131013a01320131ull, 0x13800cc005d0132ull, 0x131013a01320131ull, 0x1300131008f0130ull, 0xf6013a813000f6ull, 0xf5013a813000f5ull, 0xf7013a013000f7ull,
    0x139013901390130ull, 0x138013a005e0132ull, 0x130013a01320130ull, 0x138013000d60130ull, 0x139013901390131ull, 0x130013100900130ull, 0xf7013a813000f7ull, 0xf6013a013000f6ull,
    0xf5013a013000f5ull, 0x139013901390130ull, 0x1380057003d0132ull, 0x130013a01320130ull, 0x1380059003b0132ull, 0x130013a01320130ull, 0x138013000d70130ull, 0x139013901390131ull,
    0x13800c900570132ull, 0x131013a01320131ull, 0x13800c700590132ull, 0x131013a01320131ull, 0x130013100910130ull, 0xf0013a813000f0ull, 0xf2013a813000f2ull, 0xf5013a013000f5ull,
    0x139013901390130ull, 0x138013a00550132ull, 0x130013a01320130ull, 0x138013000d80130ull, 0x139013901390131ull, 0x130013100920130ull, 0xee013a813000eeull, 0xef013a013000efull,
    0xed013a013000edull, 0x139013901390130ull, 0x138013a00530132ull, 0x130013a01320130ull, 0x138013000d90130ull, 0x139013901390131ull, 0x130013100930130ull, 0xec013a813000ecull,
    0xf0013a013000f0ull, 0xf3013a013000f3ull, 0x139013901390130ull, 0x138013a00590132ull, 0x130013a01320130ull, 0x138013000da0130ull, 0x139013901390131ull, 0x130013100940130ull,
    0xf2013a813000f2ull, 0xf0013a013000f0ull, 0xf6013a013000f6ull, 0x139013901390130ull, 0x138013a00560132ull, 0x130013a01320130ull, 0x138013000db0130ull, 0x139013901390131ull,
    0x130013100950130ull, 0xef013a813000efull, 0xf00130013e00f0ull, 0xef00ee800800efull, 0xf000ec800a00f0ull, 0xf000ef800b00f0ull, 0xf100ed800e00f1ull, 0xf100ee800f00f1ull,
    0xf200f0801400f2ull, 0xf300ec801600f3ull, 0xf300f1801700f3ull, 0xf400ed801c00f4ull, 0xf400ee801d00f4ull, 0xf400f1801e00f4ull, 0xf400f3801f00f4ull, 0xf500f0802300f5ull,
    0xf500f1802400f5ull, 0xf500f2802500f5ull, 0xf500f3802600f5ull, 0xf500f4802700f5ull, 0xf600f1802b00f6ull, 0xf600f2802c00f6ull, 0xf600f3802d00f6ull, 0xf600f4802e00f6ull,
    0xf600f5802f00f6ull, 0xf700f5803200f7ull, 0xf700f6803300f7ull, 0x138003400f700f7ull, 0xf600f7803100f6ull, 0x138003000f600f6ull, 0xf500f6802900f5ull, 0xf500f7802a00f5ull,
    0x138002800f500f5ull, 0xf400f5802100f4ull, 0xf400f6802200f4ull, 0x138002000f400f4ull, 0xf300f4801900f3ull, 0xf300f5801a00f3ull, 0xf300f6801b00f3ull, 0x138001800f300f3ull,
    0x138001500f200f2ull, 0xf100f3801100f1ull, 0xf100f4801200f1ull, 0xf100f6801300f1ull, 0x138001000f100f1ull, 0xf000f2800d00f0ull, 0x138000c00f000f0ull, 0x138000900ef00efull,
    0x138000700ee00eeull, 0xed00ee800400edull, 0xed00f1800500edull, 0xed00f4800600edull, 0x138000300ed00edull, 0x138000200ec00ecull, 0x138000100eb00ebull, 0x138000000ea00eaull,
    0x138013a010600f8ull, 0xf800dc013c00f8ull, 0xf800ea013d00f8ull, 0x138013a010700f9ull, 0xf900dd013c00f9ull, 0xf900eb013d00f9ull, 0x138013a010800faull, 0xfa00de013c00faull,
    0xfa00ec013d00faull, 0x138013a010900fbull, 0xfb00df013c00fbull, 0xfb00ed013d00fbull, 0x138013a010a00fcull, 0xfc00e0013c00fcull, 0xfc00ee013d00fcull, 0x138013a010b00fdull,
    0xfd00e1013c00fdull, 0xfd00ef013d00fdull, 0x138013a010c00feull, 0xfe00e2013c00feull, 0xfe00f0013d00feull, 0x138013a010d00ffull, 0xff00e3013c00ffull, 0xff00f1013d00ffull,
    0x138013a010e0100ull, 0x10000e4013c0100ull, 0x10000f2013d0100ull, 0x138013a010f0101ull, 0x10100e5013c0101ull, 0x10100f3013d0101ull, 0x138013a01100102ull, 0x10200e6013c0102ull,
    0x10200f4013d0102ull, 0x138013a01110103ull, 0x10300e7013c0103ull, 0x10300f5013d0103ull, 0x138013a01120104ull, 0x10400e8013c0104ull, 0x10400f6013d0104ull, 0x138013a01130105ull,
    0x10500e9013c0105ull, 0x10500f7013d0105ull, 0x139013901390130ull, 0x138013a006b0132ull, 0x130013a01320130ull, 0x138013000cf0130ull, 0x139013901390131ull, 0x130013100890130ull,
    0x104013a81300104ull, 0x101013a01300101ull, 0x102013a01300102ull, 0x139013901390130ull, 0x1380062003f0132ull, 0x130013a01320130ull, 0x138006900380132ull, 0x130013a01320130ull,
    0x138013000d00130ull, 0x139013901390131ull, 0x13800cb00620132ull, 0x131013a01320131ull, 0x13800c400690132ull, 0x131013a01320131ull, 0x1300131008a0130ull, 0x102013a81300102ull,
    0xfb013a813000fbull, 0xff013a013000ffull, 0x139013901390130ull, 0x1380066003f0132ull, 0x130013a01320130ull, 0x1380069003c0132ull, 0x130013a01320130ull, 0x138013000d10130ull,
    0x139013901390131ull, 0x13800cb00660132ull, 0x131013a01320131ull, 0x13800c800690132ull, 0x131013a01320131ull, 0x1300131008b0130ull, 0x102013a81300102ull, 0xff013a813000ffull,
    0xfb0130013e00fbull, 0x139013901390130ull, 0x1380066003e0132ull, 0x130013a01320130ull, 0x1380068003c0132ull, 0x130013a01320130ull, 0x138013000d20130ull, 0x139013901390131ull,
    0x13800ca00660132ull, 0x131013a01320131ull, 0x13800c800680132ull, 0x131013a01320131ull, 0x1300131008c0130ull, 0xff013a813000ffull, 0x101013a81300101ull, 0x104013a01300104ull,
    0x139013901390130ull, 0x138006600410132ull, 0x130013a01320130ull, 0x138006b003c0132ull, 0x130013a01320130ull, 0x138013000d30130ull, 0x139013901390131ull, 0x13800cd00660132ull,
    0x131013a01320131ull, 0x13800c8006b0132ull, 0x131013a01320131ull, 0x1300131008d0130ull, 0xff013a813000ffull, 0x104013a81300104ull, 0x103013a01300103ull, 0x139013901390130ull,
    0x138006800400132ull, 0x130013a01320130ull, 0x138006a003e0132ull, 0x130013a01320130ull, 0x138013000d40130ull, 0x139013901390131ull, 0x13800cc00680132ull, 0x131013a01320131ull,
    0x13800ca006a0132ull, 0x131013a01320131ull, 0x1300131008e0130ull, 0x101013a81300101ull, 0x103013a81300103ull, 0x1040130013e0104ull, 0x139013901390130ull, 0x138006a00410132ull,
    0x130013a01320130ull, 0x138006b00400132ull, 0x130013a01320130ull, 0x138013000d50130ull, 0x139013901390131ull, 0x13800cd006a0132ull, 0x131013a01320131ull, 0x13800cc006b0132ull,
    0x131013a01320131ull, 0x1300131008f0130ull, 0x104013a81300104ull, 0x103013a81300103ull, 0x105013a01300105ull, 0x139013901390130ull, 0x138013a006c0132ull, 0x130013a01320130ull,
    0x138013000d60130ull, 0x139013901390131ull, 0x130013100900130ull, 0x105013a81300105ull, 0x104013a01300104ull, 0x103013a01300103ull, 0x139013901390130ull, 0x1380065003d0132ull,
    0x130013a01320130ull, 0x1380067003b0132ull, 0x130013a01320130ull, 0x138013000d70130ull, 0x139013901390131ull, 0x13800c900650132ull, 0x131013a01320131ull, 0x13800c700670132ull,
    0x131013a01320131ull, 0x130013100910130ull, 0xfe013a813000feull, 0x100013a81300100ull, 0x103013a01300103ull, 0x139013901390130ull, 0x138013a00630132ull, 0x130013a01320130ull,
    0x138013000d80130ull, 0x139013901390131ull, 0x130013100920130ull, 0xfc013a813000fcull, 0xfd013a013000fdull, 0xfb013a013000fbull, 0x139013901390130ull, 0x138013a00610132ull,
    0x130013a01320130ull, 0x138013000d90130ull, 0x139013901390131ull, 0x130013100930130ull, 0xfa013a813000faull, 0xfe013a013000feull, 0x101013a01300101ull, 0x139013901390130ull,
    0x138013a00670132ull, 0x130013a01320130ull, 0x138013000da0130ull, 0x139013901390131ull, 0x130013100940130ull, 0x100013a81300100ull, 0xfe013a013000feull, 0x104013a01300104ull,
    0x139013901390130ull, 0x138013a00640132ull, 0x130013a01320130ull, 0x138013000db0130ull, 0x139013901390131ull, 0x130013100950130ull, 0xfd013a813000fdull, 0xfe0130013e00feull,
    0xfd00fc800800fdull, 0xfe00fa800a00feull, 0xfe00fd800b00feull, 0xff00fb800e00ffull, 0xff00fc800f00ffull, 0x10000fe80140100ull, 0x10100fa80160101ull, 0x10100ff80170101ull,
    0x10200fb801c0102ull, 0x10200fc801d0102ull, 0x10200ff801e0102ull, 0x1020101801f0102ull, 0x10300fe80230103ull, 0x10300ff80240103ull, 0x103010080250103ull, 0x103010180260103ull,
    0x103010280270103ull, 0x10400ff802b0104ull, 0x1040100802c0104ull, 0x1040101802d0104ull, 0x1040102802e0104ull, 0x1040103802f0104ull, 0x105010380320105ull, 0x105010480330105ull,
    0x138003401050105ull, 0x104010580310104ull, 0x138003001040104ull, 0x103010480290103ull, 0x1030105802a0103ull, 0x138002801030103ull, 0x102010380210102ull, 0x102010480220102ull,
    0x138002001020102ull, 0x101010280190101ull, 0x1010103801a0101ull, 0x1010104801b0101ull, 0x138001801010101ull, 0x138001501000100ull, 0xff0101801100ffull, 0xff0102801200ffull,
    0xff0104801300ffull, 0x138001000ff00ffull, 0xfe0100800d00feull, 0x138000c00fe00feull, 0x138000900fd00fdull, 0x138000700fc00fcull, 0xfb00fc800400fbull, 0xfb00ff800500fbull,
    0xfb0102800600fbull, 0x138000300fb00fbull, 0x138000200fa00faull, 0x138000100f900f9ull, 0x138000000f800f8ull, 0xc1013a00dc00c1ull, 0xc100ea013f00c1ull, 0xc100f8014000c1ull,
    0xc2013a00dd00c2ull, 0xc200eb013f00c2ull, 0xc200f9014000c2ull, 0xc3013a00de00c3ull, 0xc300ec013f00c3ull, 0xc300fa014000c3ull, 0xc4013a00df00c4ull, 0xc400ed013f00c4ull,
    0xc400fb014000c4ull, 0xc5013a00e000c5ull, 0xc500ee013f00c5ull, 0xc500fc014000c5ull, 0xc6013a00e100c6ull, 0xc600ef013f00c6ull, 0xc600fd014000c6ull, 0xc7013a00e200c7ull,
    0xc700f0013f00c7ull, 0xc700fe014000c7ull, 0xc8013a00e300c8ull, 0xc800f1013f00c8ull, 0xc800ff014000c8ull, 0xc9013a00e400c9ull, 0xc900f2013f00c9ull, 0xc90100014000c9ull,
    0xca013a00e500caull, 0xca00f3013f00caull, 0xca0101014000caull, 0xcb013a00e600cbull, 0xcb00f4013f00cbull, 0xcb0102014000cbull, 0xcc013a00e700ccull, 0xcc00f5013f00ccull,
    0xcc0103014000ccull, 0xcd013a00e800cdull, 0xcd00f6013f00cdull, 0xcd0104014000cdull, 0xce013a00e900ceull, 0xce00f7013f00ceull, 0xce0105014000ceull,
};
}  // namespace coop


struct Mech {
  static constexpr const char* NAME = "saprc99_mini";
  static constexpr int NS = 17;      // species including fixed ones
  static constexpr int NV = 14;      // variable species (solved system)
  static constexpr int NR = 13;      // reactions
  static constexpr int NP = 4;      // runtime parameter slots per cell
  static constexpr int NPH = 4;      // photolysis slots
  static constexpr int NFIX = 3;
  static constexpr int NLU = 53;
  static constexpr int NSTAGE = 3;
  static constexpr bool RUNTIME_ENV = true;
  static constexpr bool CLOUD_GATED = false;
  static constexpr double GAMMA = 0.435866521508459;
  static constexpr double ELO = 3.0;
  static constexpr double SEED = 9.9999999999999995e-07;
  static constexpr double ENV_T = 298.14999999999998;
  static constexpr double ENV_RHO = 2.46e+19;
  static constexpr long long LU_FMA = 38;
  static constexpr long long LU_SCALE = 24;
  static constexpr long long SOLVE_L = 24;
  static constexpr long long SOLVE_U = 15;
  static constexpr long long FUN_FLOPS = 96;
  static constexpr long long JAC_FLOPS = 132;

  __host__ __device__ static constexpr int var_phys(int i) { constexpr int t[14] = {14, 8, 6, 13, 11, 1, 10, 0, 7, 2, 9, 4, 3, 5}; return t[i]; }
  __host__ __device__ static constexpr int fix_phys(int i) { constexpr int t[3] = {12, 15, 16}; return t[i]; }
  __host__ __device__ static constexpr double atol_v(int i) { constexpr double t[14] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0}; return t[i]; }
  __host__ __device__ static constexpr double rtol_v(int i) { constexpr double t[14] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001}; return t[i]; }
  static constexpr double ATOL[NS] = {1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0, 1.0};
  static constexpr double RTOL[NS] = {0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001, 0.001};
  __host__ __device__ static constexpr int lu_prow(int s) { constexpr int t[53] = {14, 8, 6, 13, 13, 13, 13, 11, 1, 1, 10, 10, 10, 10, 0, 0, 0, 0, 0, 0, 7, 7, 2, 2, 2, 2, 2, 2, 9, 9, 9, 9, 9, 9, 9, 4, 4, 4, 4, 4, 4, 4, 4, 3, 3, 3, 3, 3, 3, 3, 5, 5, 5}; return t[s]; }
  __host__ __device__ static constexpr int lu_pcol(int s) { constexpr int t[53] = {14, 8, 6, 13, 11, 0, 9, 11, 11, 1, 6, 1, 10, 7, 13, 11, 0, 2, 9, 3, 10, 7, 6, 0, 2, 9, 4, 3, 13, 11, 0, 2, 9, 4, 3, 10, 0, 7, 2, 9, 4, 3, 5, 0, 7, 2, 9, 4, 3, 5, 4, 3, 5}; return t[s]; }
  static const char* species_name(int s) { static const char* t[17] = {"O3", "H2O2", "NO", "NO2", "NO3", "N2O5", "HONO", "HNO3", "HNO4", "O3P", "OH", "HO2", "AIR", "O2", "H2O", "M", "N2"}; return t[s]; }
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
    k.set(1, 4.9010355073084971e-27*pow(T, -2.7999999999999998)*FIX(12));
    k.set(2, 7.9999999999999998e-12*exp(-2060.0/T));
    k.set(3, 1.8e-12*exp(-1370.0/T));
    k.set(4, 1.4000000000000001e-13*exp(-2470.0/T));
    k.set(5, 1.7999999999999999e-11*exp(110.0/T));
    k.set(6, 2.7999999999999999e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*FIX(12)*exp(3.5/T)/(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0));
    k.set(7, 2.1383343303319472e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*FIX(12)*exp(11000.0/T)/(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0));
    k.set(8, 1.9e-33*FIX(12)*exp(725.0/T)/(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0) + 7.2000000000000002e-15*exp(785.0/T));
    k.set(9, 1.7e-33*FIX(12)*exp(1000.0/T) + 2.2999999999999998e-13*exp(600.0/T));
    k.set(10, P(1));
    k.set(11, P(2));
    k.set(12, P(3));
  }

  // Per-cell working storage, in slots of one double: the LU factors, the
  // state y, the stage vectors K_1..K_s, the tendency F, the increment dy and
  // the rate constants of the current host step.
  static constexpr int Y = 53;
  static constexpr int K0 = 67;
  static constexpr int F = 109;
  static constexpr int DY = 123;
  static constexpr int KT = 137;        // the cell's rate constants for the current host step
  static constexpr int NSLOTS = 150;
  static constexpr bool TABLE_ATTEMPT = false;

  // Mass-action tendencies F(y) of the variable species (logical order):
  // y(i) supplies the state, out(i, F_i) receives the result.
  template <class YA, class KA, class FO>
  __device__ __noinline__ static void fun(const YA& y, const KA& k, FO&& out) {
    const double y2 = y(2);
    const double y3 = y(3);
    const double y4 = y(4);
    const double y5 = y(5);
    const double y6 = y(6);
    const double y7 = y(7);
    const double y8 = y(8);
    const double y9 = y(9);
    const double y10 = y(10);
    const double y11 = y(11);
    const double y12 = y(12);
    const double y13 = y(13);
    const double q0 = k(0) * y12;
    const double q1 = k(1) * y10 * y3;
    const double q2 = k(2) * y10 * y7;
    const double q3 = k(3) * y7 * y9;
    const double q4 = k(4) * y7 * y12;
    const double q5 = k(5) * y9 * y11;
    const double q6 = k(6) * y12 * y11;
    const double q7 = k(7) * y13;
    const double q8 = k(8) * y6 * y8;
    const double q9 = k(9) * y4;
    const double q10 = k(10) * y2;
    const double q11 = k(11) * y8;
    const double q12 = k(12) * y5;
    out(0, 0.0);
    out(1, 0.0);
    out(2, -q10);
    out(3, fma(2.0, q2, -q1) + q9);
    out(4, -q9);
    out(5, q9 - q12);
    out(6, fma(2.0, q12, -q8 + q10 + q11));
    out(7, q1 - q2 - q3 - q4);
    out(8, -q8 - q11);
    out(9, q0 - q3 - q5 + q10);
    out(10, q0 - q1 - q2);
    out(11, q4 - q5 - q6 + q7 + q8);
    out(12, fma(2.0, q5, -q0 + q3 - q4) - q6 + q7 + q11);
    out(13, q6 - q7);
  }

  // W = I/(gamma h) - J(y) into the LU slots that hold W entries.
  template <class YA, class KA, class SA>
  __device__ __noinline__ static void jac_w(const YA& y, const KA& k, double inv_g_dt, SA& S) {
    (void)inv_g_dt;
    const double y3 = y(3);
    const double y6 = y(6);
    const double y7 = y(7);
    const double y8 = y(8);
    const double y9 = y(9);
    const double y10 = y(10);
    const double y11 = y(11);
    const double y12 = y(12);
    const double d0_12 = k(0);
    const double d1_10 = k(1) * y3;
    const double d1_3 = k(1) * y10;
    const double d2_10 = k(2) * y7;
    const double d2_7 = k(2) * y10;
    const double d3_7 = k(3) * y9;
    const double d3_9 = k(3) * y7;
    const double d4_7 = k(4) * y12;
    const double d4_12 = k(4) * y7;
    const double d5_9 = k(5) * y11;
    const double d5_11 = k(5) * y9;
    const double d6_12 = k(6) * y11;
    const double d6_11 = k(6) * y12;
    const double d7_13 = k(7);
    const double d8_6 = k(8) * y8;
    const double d8_8 = k(8) * y6;
    const double d9_4 = k(9);
    const double d10_2 = k(10);
    const double d11_8 = k(11);
    const double d12_5 = k(12);
    S[0] = inv_g_dt;
    S[1] = inv_g_dt;
    S[2] = inv_g_dt + d10_2;
    S[3] = inv_g_dt + d1_3;
    S[4] = -d9_4;
    S[5] = -2.0 * d2_7;
    S[6] = fma(-2.0, d2_10, d1_10);
    S[7] = inv_g_dt + d9_4;
    S[8] = -d9_4;
    S[9] = inv_g_dt + d12_5;
    S[10] = -d10_2;
    S[11] = -2.0 * d12_5;
    S[12] = inv_g_dt + d8_6;
    S[13] = d8_8 - d11_8;
    S[14] = -d1_3;
    S[16] = inv_g_dt + d2_7 + d3_7 + d4_7;
    S[17] = d3_9;
    S[18] = -d1_10 + d2_10;
    S[19] = d4_12;
    S[20] = d8_6;
    S[21] = inv_g_dt + d8_8 + d11_8;
    S[22] = -d10_2;
    S[23] = d3_7;
    S[24] = inv_g_dt + d3_9 + d5_9;
    S[26] = d5_11;
    S[27] = -d0_12;
    S[28] = d1_3;
    S[30] = d2_7;
    S[32] = inv_g_dt + d1_10 + d2_10;
    S[34] = -d0_12;
    S[35] = -d8_6;
    S[36] = -d4_7;
    S[37] = -d8_8;
    S[38] = d5_9;
    S[40] = inv_g_dt + d5_11 + d6_11;
    S[41] = -d4_12 + d6_12;
    S[42] = -d7_13;
    S[43] = -d3_7 + d4_7;
    S[44] = -d11_8;
    S[45] = fma(-2.0, d5_9, -d3_9);
    S[47] = -2.0 * d5_11 + d6_11;
    S[48] = inv_g_dt + d0_12 + d4_12 + d6_12;
    S[49] = -d7_13;
    S[50] = -d6_11;
    S[51] = -d6_12;
    S[52] = inv_g_dt + d7_13;
  }

  // Physical (row, column) of every W slot, for the dense Jacobian.
  template <class Fn>
  __device__ __forceinline__ static void for_each_w_slot(Fn&& fn) {
    fn(0, 14, 14);
    fn(1, 8, 8);
    fn(2, 6, 6);
    fn(3, 13, 13);
    fn(4, 13, 11);
    fn(5, 13, 0);
    fn(6, 13, 9);
    fn(7, 11, 11);
    fn(8, 1, 11);
    fn(9, 1, 1);
    fn(10, 10, 6);
    fn(11, 10, 1);
    fn(12, 10, 10);
    fn(13, 10, 7);
    fn(14, 0, 13);
    fn(16, 0, 0);
    fn(17, 0, 2);
    fn(18, 0, 9);
    fn(19, 0, 3);
    fn(20, 7, 10);
    fn(21, 7, 7);
    fn(22, 2, 6);
    fn(23, 2, 0);
    fn(24, 2, 2);
    fn(26, 2, 4);
    fn(27, 2, 3);
    fn(28, 9, 13);
    fn(30, 9, 0);
    fn(32, 9, 9);
    fn(34, 9, 3);
    fn(35, 4, 10);
    fn(36, 4, 0);
    fn(37, 4, 7);
    fn(38, 4, 2);
    fn(40, 4, 4);
    fn(41, 4, 3);
    fn(42, 4, 5);
    fn(43, 3, 0);
    fn(44, 3, 7);
    fn(45, 3, 2);
    fn(47, 3, 4);
    fn(48, 3, 3);
    fn(49, 3, 5);
    fn(50, 5, 4);
    fn(51, 5, 3);
    fn(52, 5, 5);
  }

  // Fixed-species columns of the dense Jacobian: dF_i/dC_f through the
  // rate constants' dependence on fixed species (third bodies).
  template <class PA, class FA, class YA, class Fn>
  __device__ __forceinline__ static void jac_fixed_columns(const PA& P, const FA& FIX, double T, double RHO,
                                                         double RH, double CLW, const YA& y, Fn&& fn) {
    (void)T; (void)RHO; (void)RH; (void)CLW; (void)P; (void)FIX; (void)y;
    fn(0, 12, ((4.9010355073084971e-27*pow(T, -2.7999999999999998)) * y(10) * y(3)));
    fn(1, 12, ((1.7e-33*exp(1000.0/T)) * y(4)));
    fn(3, 12, -((-3.9199999999999996e-48*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*FIX(12)*exp(7.2000000000000002/T)/pow(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0, 2) + 2.7999999999999999e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)/(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0) + 4.4716430988195204e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)*log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T))/((1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0)*pow(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*pow(M_LN10, 2))) * y(12) * y(11)) + ((2.1383343303319472e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)/(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0) + 3.4149528397134688e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)*log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T))/(pow(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0)*pow(M_LN10, 2)) - 2.6648167974096755e-39*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 7.0999999999999996)*FIX(12)*exp(10920.0/T)/pow(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0, 2)) * y(13)));
    fn(4, 12, -((-3.9199999999999996e-48*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*FIX(12)*exp(7.2000000000000002/T)/pow(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0, 2) + 2.7999999999999999e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)/(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0) + 4.4716430988195204e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)*log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T))/((1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0)*pow(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*pow(M_LN10, 2))) * y(12) * y(11)) + ((2.1383343303319472e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)/(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0) + 3.4149528397134688e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)*log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T))/(pow(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0)*pow(M_LN10, 2)) - 2.6648167974096755e-39*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 7.0999999999999996)*FIX(12)*exp(10920.0/T)/pow(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0, 2)) * y(13)) + ((-8.8048780487804873e-51*FIX(12)*exp(10.0/T)/pow(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0, 2) + 1.9e-33*exp(725.0/T)/(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0)) * y(6) * y(8)));
    fn(5, 12, ((-3.9199999999999996e-48*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*FIX(12)*exp(7.2000000000000002/T)/pow(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0, 2) + 2.7999999999999999e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)/(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0) + 4.4716430988195204e-30*pow(0.45000000000000001, 1.0/(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0))*exp(3.5/T)*log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T))/((1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T) + 1.0)*pow(pow(log(1.3999999999999999e-18*FIX(12)*exp(3.7000000000000002/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*pow(M_LN10, 2))) * y(12) * y(11)) - ((2.1383343303319472e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)/(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0) + 3.4149528397134688e-12*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 3.5)*exp(11000.0/T)*log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T))/(pow(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0, 2)*(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0)*pow(M_LN10, 2)) - 2.6648167974096755e-39*pow(0.45000000000000001, 1.0/(pow(log(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T)), 2)/pow(M_LN10, 2) + 1.0))*pow(T, 7.0999999999999996)*FIX(12)*exp(10920.0/T)/pow(1.2462114832136653e-27*pow(T, 3.6000000000000001)*FIX(12)*exp(-80.0/T) + 1.0, 2)) * y(13)));
    fn(7, 12, -((-8.8048780487804873e-51*FIX(12)*exp(10.0/T)/pow(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0, 2) + 1.9e-33*exp(725.0/T)/(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0)) * y(6) * y(8)));
    fn(9, 12, -((4.9010355073084971e-27*pow(T, -2.7999999999999998)) * y(10) * y(3)));
    fn(10, 12, -((-8.8048780487804873e-51*FIX(12)*exp(10.0/T)/pow(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0, 2) + 1.9e-33*exp(725.0/T)/(4.6341463414634146e-18*FIX(12)*exp(-715.0/T) + 1.0)) * y(6) * y(8)));
    fn(11, 12, -((1.7e-33*exp(1000.0/T)) * y(4)));
    fn(13, 12, -((4.9010355073084971e-27*pow(T, -2.7999999999999998)) * y(10) * y(3)) + ((1.7e-33*exp(1000.0/T)) * y(4)));
  }

  // In-place row-wise Doolittle LU over the compact slots, in the operation
  // order of the reference plan.  The operands a row reuses (its own L
  // entries for the U part, the pivot column of U for the L part) are read
  // once into registers.  Diagonal slots end up holding 1/U_ii.
  template <class SA>
  __device__ __noinline__ static bool factor(SA& S) {
    bool ok = true;
    {  // pivot row 0
      const double u0 = S[0];
      ok = ok && (u0 != 0.0);
      const double rd = 1.0 / u0;
      S[0] = rd;
    }
    {  // pivot row 1
      const double u1 = S[1];
      ok = ok && (u1 != 0.0);
      const double rd = 1.0 / u1;
      S[1] = rd;
    }
    {  // pivot row 2
      const double u2 = S[2];
      ok = ok && (u2 != 0.0);
      const double rd = 1.0 / u2;
      S[2] = rd;
      double v10 = S[10];
      double v22 = S[22];
      S[10] = v10 * rd;
      S[22] = v22 * rd;
    }
    {  // pivot row 3
      const double u3 = S[3];
      ok = ok && (u3 != 0.0);
      const double rd = 1.0 / u3;
      S[3] = rd;
      double v4 = S[4];
      double v5 = S[5];
      double v6 = S[6];
      double v14 = S[14];
      double v28 = S[28];
      S[14] = v14 * rd;
      S[28] = v28 * rd;
    }
    {  // pivot row 4
      const double u7 = S[7];
      ok = ok && (u7 != 0.0);
      const double rd = 1.0 / u7;
      S[7] = rd;
      const double b4 = S[4];
      double v8 = S[8];
      double v15 = 0.0;
      double v29 = 0.0;
      v15 = fma(-S[14], b4, v15);
      v29 = fma(-S[28], b4, v29);
      S[8] = v8 * rd;
      S[15] = v15 * rd;
      S[29] = v29 * rd;
    }
    {  // pivot row 5
      const double u9 = S[9];
      ok = ok && (u9 != 0.0);
      const double rd = 1.0 / u9;
      S[9] = rd;
      double v11 = S[11];
      S[11] = v11 * rd;
    }
    {  // pivot row 6
      const double u12 = S[12];
      ok = ok && (u12 != 0.0);
      const double rd = 1.0 / u12;
      S[12] = rd;
      double v13 = S[13];
      double v20 = S[20];
      double v35 = S[35];
      S[20] = v20 * rd;
      S[35] = v35 * rd;
    }
    {  // pivot row 7
      const double a14 = S[14];
      const double u16 = fma(-a14, S[5], S[16]);
      ok = ok && (u16 != 0.0);
      const double rd = 1.0 / u16;
      S[16] = rd;
      double v17 = S[17];
      double v18 = S[18];
      double v19 = S[19];
      v18 = fma(-a14, S[6], v18);
      S[18] = v18;
      const double b5 = S[5];
      double v23 = S[23];
      double v30 = S[30];
      double v36 = S[36];
      double v43 = S[43];
      v30 = fma(-S[28], b5, v30);
      S[23] = v23 * rd;
      S[30] = v30 * rd;
      S[36] = v36 * rd;
      S[43] = v43 * rd;
    }
    {  // pivot row 8
      const double a20 = S[20];
      const double u21 = fma(-a20, S[13], S[21]);
      ok = ok && (u21 != 0.0);
      const double rd = 1.0 / u21;
      S[21] = rd;
      const double b13 = S[13];
      double v37 = S[37];
      double v44 = S[44];
      v37 = fma(-S[35], b13, v37);
      S[37] = v37 * rd;
      S[44] = v44 * rd;
    }
    {  // pivot row 9
      const double a23 = S[23];
      const double u24 = fma(-a23, S[17], S[24]);
      ok = ok && (u24 != 0.0);
      const double rd = 1.0 / u24;
      S[24] = rd;
      double v25 = 0.0;
      double v26 = S[26];
      double v27 = S[27];
      v25 = fma(-a23, S[18], v25);
      v27 = fma(-a23, S[19], v27);
      S[25] = v25;
      S[27] = v27;
      const double b17 = S[17];
      double v31 = 0.0;
      double v38 = S[38];
      double v45 = S[45];
      v31 = fma(-S[30], b17, v31);
      v38 = fma(-S[36], b17, v38);
      v45 = fma(-S[43], b17, v45);
      S[31] = v31 * rd;
      S[38] = v38 * rd;
      S[45] = v45 * rd;
    }
    {  // pivot row 10
      const double a28 = S[28];
      const double a30 = S[30];
      const double a31 = S[31];
      const double u32 = fma(-a31, S[25], fma(-a30, S[18], fma(-a28, S[6], S[32])));
      ok = ok && (u32 != 0.0);
      const double rd = 1.0 / u32;
      S[32] = rd;
      double v33 = 0.0;
      double v34 = S[34];
      v33 = fma(-a31, S[26], v33);
      v34 = fma(-a30, S[19], v34);
      v34 = fma(-a31, S[27], v34);
      S[33] = v33;
      S[34] = v34;
      const double b18 = S[18];
      const double b25 = S[25];
      double v39 = 0.0;
      double v46 = 0.0;
      v39 = fma(-S[36], b18, v39);
      v46 = fma(-S[43], b18, v46);
      v39 = fma(-S[38], b25, v39);
      v46 = fma(-S[45], b25, v46);
      S[39] = v39 * rd;
      S[46] = v46 * rd;
    }
    {  // pivot row 11
      const double a36 = S[36];
      const double a38 = S[38];
      const double a39 = S[39];
      const double u40 = fma(-a39, S[33], fma(-a38, S[26], S[40]));
      ok = ok && (u40 != 0.0);
      const double rd = 1.0 / u40;
      S[40] = rd;
      double v41 = S[41];
      double v42 = S[42];
      v41 = fma(-a36, S[19], v41);
      v41 = fma(-a38, S[27], v41);
      v41 = fma(-a39, S[34], v41);
      S[41] = v41;
      const double b26 = S[26];
      const double b33 = S[33];
      double v47 = S[47];
      double v50 = S[50];
      v47 = fma(-S[45], b26, v47);
      v47 = fma(-S[46], b33, v47);
      S[47] = v47 * rd;
      S[50] = v50 * rd;
    }
    {  // pivot row 12
      const double a43 = S[43];
      const double a45 = S[45];
      const double a46 = S[46];
      const double a47 = S[47];
      const double u48 = fma(-a47, S[41], fma(-a46, S[34], fma(-a45, S[27], fma(-a43, S[19], S[48]))));
      ok = ok && (u48 != 0.0);
      const double rd = 1.0 / u48;
      S[48] = rd;
      double v49 = S[49];
      v49 = fma(-a47, S[42], v49);
      S[49] = v49;
      const double b41 = S[41];
      double v51 = S[51];
      v51 = fma(-S[50], b41, v51);
      S[51] = v51 * rd;
    }
    {  // pivot row 13
      const double a50 = S[50];
      const double a51 = S[51];
      const double u52 = fma(-a51, S[49], fma(-a50, S[42], S[52]));
      ok = ok && (u52 != 0.0);
      const double rd = 1.0 / u52;
      S[52] = rd;
    }
    return ok;
  }

  // Solve (LU) x = b in place on slots [base, base + NV): unit-L forward
  // sweep, then the U backward sweep scaled by the stored 1/U_ii.
  template <class SA>
  __device__ __noinline__ static void solve(SA& S, const int base) {
    const double v0 = S[base + 0];
    const double v1 = S[base + 1];
    const double v2 = S[base + 2];
    const double v3 = S[base + 3];
    const double v4 = S[base + 4];
    const double v5 = fma(-S[8], v4, S[base + 5]);
    const double v6 = fma(-S[11], v5, fma(-S[10], v2, S[base + 6]));
    const double v7 = fma(-S[15], v4, fma(-S[14], v3, S[base + 7]));
    const double v8 = fma(-S[20], v6, S[base + 8]);
    const double v9 = fma(-S[23], v7, fma(-S[22], v2, S[base + 9]));
    const double v10 = fma(-S[31], v9, fma(-S[30], v7, fma(-S[29], v4, fma(-S[28], v3, S[base + 10]))));
    const double v11 = fma(-S[39], v10, fma(-S[38], v9, fma(-S[37], v8, fma(-S[36], v7, fma(-S[35], v6, S[base + 11])))));
    const double v12 = fma(-S[47], v11, fma(-S[46], v10, fma(-S[45], v9, fma(-S[44], v8, fma(-S[43], v7, S[base + 12])))));
    const double v13 = fma(-S[51], v12, fma(-S[50], v11, S[base + 13]));
    const double x13 = (v13) * S[52];
    S[base + 13] = x13;
    const double x12 = (fma(-S[49], x13, v12)) * S[48];
    S[base + 12] = x12;
    const double x11 = (fma(-S[42], x13, fma(-S[41], x12, v11))) * S[40];
    S[base + 11] = x11;
    const double x10 = (fma(-S[34], x12, fma(-S[33], x11, v10))) * S[32];
    S[base + 10] = x10;
    const double x9 = (fma(-S[27], x12, fma(-S[26], x11, fma(-S[25], x10, v9)))) * S[24];
    S[base + 9] = x9;
    const double x8 = (v8) * S[21];
    S[base + 8] = x8;
    const double x7 = (fma(-S[19], x12, fma(-S[18], x10, fma(-S[17], x9, v7)))) * S[16];
    S[base + 7] = x7;
    const double x6 = (fma(-S[13], x8, v6)) * S[12];
    S[base + 6] = x6;
    const double x5 = (v5) * S[9];
    S[base + 5] = x5;
    const double x4 = (v4) * S[7];
    S[base + 4] = x4;
    const double x3 = (fma(-S[6], x10, fma(-S[5], x7, fma(-S[4], x4, v3)))) * S[3];
    S[base + 3] = x3;
    const double x2 = (v2) * S[2];
    S[base + 2] = x2;
    const double x1 = (v1) * S[1];
    S[base + 1] = x1;
    const double x0 = (v0) * S[0];
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
      S[67 + i] = S[F + i];
    }
    solve(S, 67);
    fun([&](int i) { return S[Y + i] + S[67 + i]; }, k, [&](int i, double v) { S[F + i] = v; });
    const double c21 = -1.0156171083877703 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[81 + i] = fma(c21, S[67 + i], S[F + i]);
    }
    solve(S, 81);
    const double c31 = 4.0759956452537702 / h;
    const double c32 = 9.20767942983308 / h;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      S[95 + i] = fma(c32, S[81 + i], fma(c31, S[67 + i], S[F + i]));
    }
    solve(S, 95);
    double err_sq = 0.0;
    #pragma unroll
    for (int i = 0; i < NV; ++i) {
      const double k0 = S[67 + i];
      const double k1 = S[81 + i];
      const double k2 = S[95 + i];
      const double yi = S[Y + i];
      const double ynew = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, yi + k0));
      S[DY + i] = fma(-0.42772256543218573, k2, fma(6.1697947043828245, k1, k0));
      const double sc = fma(rtol_v(i), fmax(fabs(yi), fabs(ynew)), atol_v(i));
      const double q = (fma(0.22354069897811571, k2, fma(-2.9079558716805471, k1, 0.5 * k0))) / sc;
      err_sq = fma(q, q, err_sq);
    }
    return fmax(sqrt(err_sq / 17.0), 1.0e-10);
  }

  // Step-size factor from the error norm (integrate.j2:324-333).
  __device__ __forceinline__ static double growth(double err) {
    const double fac = 0.9 / cbrt(err);
    return fmax(0.2, fmin(fac, 6.0));
  }

  // ---- warp-cooperative attempt (static warp schedules) ----
  static constexpr int NPART = 20;
  static constexpr int Q = 150;            // rates q_r, then q_i of the error norm
  static constexpr int D = 164;     // partial derivatives
  static constexpr int CB = 184;        // constants
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
      S[188] = -1.0156171083877703 / h;    // c21 / h
      S[189] = 4.0759956452537702 / h;    // c31 / h
      S[190] = 9.20767942983308 / h;    // c32 / h
    }
    __syncwarp();
    bool ok = true;
    for (int st = 0; st < NSTAGE; ++st) ok = run_schedule(S, T::stage_step[st], T::stage_step[st + 1], lane) && ok;
    if (__any_sync(0xffffffffu, !ok)) status |= 1;
    // Increment, and q_i^2 of the error norm into the rate slots.
    for (int i = lane; i < NV; i += 32) {
      const double k0 = S[67 + i];
      const double k1 = S[81 + i];
      const double k2 = S[95 + i];
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
      err = fmax(sqrt(err_sq / 17.0), 1.0e-10);
    }
    return __shfl_sync(0xffffffffu, err, 0);
  }

  // ---- tangent of one accepted step (forward sensitivities) ----
  static constexpr int DYT = 193;     // dy in, dy_new out (NV)
  static constexpr int DKR = 207;     // dk, the rate constants' tangent (NR)
  static constexpr int TLM_CB = 312;  // constants of the tangent program
  static constexpr int TLM_NCONST = 9;
  static constexpr int NSLOTS_TLM = 321;
  // dy_new = d(y_new)/d(y, k) (dy, dk) for one step of size h: walks
  // coop::tlm_prog.  Requires attempt() for this step first (the LU of W and
  // the K_i), y_n in S[Y..], dy in S[DYT..] and dk in S[DKR..].
  template <class SA, class KA>
  __device__ __forceinline__ static void tlm_step(SA& S, const KA& k, double h) {
    for (int r = 0; r < NR; ++r) S[KT + r] = k(r);
    for (int i = 0; i < TLM_NCONST; ++i) S[TLM_CB + i] = coop::tlm_const_val[i];
    S[315] = -1.0156171083877703 / h;    // c21 / h
    S[316] = 4.0759956452537702 / h;    // c31 / h
    S[317] = 9.20767942983308 / h;    // c32 / h
    for (int n = 0; n < coop::TLM_OPS; ++n) {
      const unsigned long long w = __ldg(coop::tlm_prog + n);
      const unsigned lo = (unsigned)w, hi = (unsigned)(w >> 32);
      const double a = __longlong_as_double(__double_as_longlong(S[(lo >> 16) & 0x7fffu]) ^
                                            ((long long)(lo >> 31) << 63));
      S[lo & 0xffffu] = fma(a, S[hi & 0xffffu], S[(hi >> 16) & 0x7fffu]);
    }
  }

  // ---- discrete adjoint of one accepted step ----
  static constexpr int LAM = 150;      // dL/dy
  static constexpr int KBAR = 164;    // stage adjoints, NSTAGE x NV
  static constexpr int FBAR = 206;    // adjoint of the pending stage tendency
  static constexpr int KB = 220;        // dL/dk accumulated
  static constexpr int NSLOTS_ADJ = 233;
  // Solve W^T x = b in place on [base, base + NV) with the stored LU of W.
  template <class SA>
  __device__ __noinline__ static void solve_t(SA& S, const int base) {
    const double z0 = (S[base + 0]) * S[0];
    const double z1 = (S[base + 1]) * S[1];
    const double z2 = (S[base + 2]) * S[2];
    const double z3 = (S[base + 3]) * S[3];
    const double z4 = (fma(-S[4], z3, S[base + 4])) * S[7];
    const double z5 = (S[base + 5]) * S[9];
    const double z6 = (S[base + 6]) * S[12];
    const double z7 = (fma(-S[5], z3, S[base + 7])) * S[16];
    const double z8 = (fma(-S[13], z6, S[base + 8])) * S[21];
    const double z9 = (fma(-S[17], z7, S[base + 9])) * S[24];
    const double z10 = (fma(-S[25], z9, fma(-S[18], z7, fma(-S[6], z3, S[base + 10])))) * S[32];
    const double z11 = (fma(-S[33], z10, fma(-S[26], z9, S[base + 11]))) * S[40];
    const double z12 = (fma(-S[41], z11, fma(-S[34], z10, fma(-S[27], z9, fma(-S[19], z7, S[base + 12]))))) * S[48];
    const double z13 = (fma(-S[49], z12, fma(-S[42], z11, S[base + 13]))) * S[52];
    const double x13 = z13;
    S[base + 13] = x13;
    const double x12 = fma(-S[51], x13, z12);
    S[base + 12] = x12;
    const double x11 = fma(-S[50], x13, fma(-S[47], x12, z11));
    S[base + 11] = x11;
    const double x10 = fma(-S[46], x12, fma(-S[39], x11, z10));
    S[base + 10] = x10;
    const double x9 = fma(-S[45], x12, fma(-S[38], x11, fma(-S[31], x10, z9)));
    S[base + 9] = x9;
    const double x8 = fma(-S[44], x12, fma(-S[37], x11, z8));
    S[base + 8] = x8;
    const double x7 = fma(-S[43], x12, fma(-S[36], x11, fma(-S[30], x10, fma(-S[23], x9, z7))));
    S[base + 7] = x7;
    const double x6 = fma(-S[35], x11, fma(-S[20], x8, z6));
    S[base + 6] = x6;
    const double x5 = fma(-S[11], x6, z5);
    S[base + 5] = x5;
    const double x4 = fma(-S[29], x10, fma(-S[15], x7, fma(-S[8], x5, z4)));
    S[base + 4] = x4;
    const double x3 = fma(-S[28], x10, fma(-S[14], x7, z3));
    S[base + 3] = x3;
    const double x2 = fma(-S[22], x9, fma(-S[10], x6, z2));
    S[base + 2] = x2;
    const double x1 = z1;
    S[base + 1] = x1;
    const double x0 = z0;
    S[base + 0] = x0;
  }

  // u^T J(y) v terms of stage i: y in S[Y..], u in S[ub..], v = K_i in S[vb..].
  template <class SA, class KA>
  __device__ __noinline__ static void adj_wterm(SA& S, const KA& k, const int ub, const int vb) {
    auto u = [&](int i) { return S[ub + i]; };
    const double y2 = S[Y + 2];
    const double v2 = S[vb + 2];
    const double y3 = S[Y + 3];
    const double v3 = S[vb + 3];
    const double y4 = S[Y + 4];
    const double v4 = S[vb + 4];
    const double y5 = S[Y + 5];
    const double v5 = S[vb + 5];
    const double y6 = S[Y + 6];
    const double v6 = S[vb + 6];
    const double y7 = S[Y + 7];
    const double v7 = S[vb + 7];
    const double y8 = S[Y + 8];
    const double v8 = S[vb + 8];
    const double y9 = S[Y + 9];
    const double v9 = S[vb + 9];
    const double y10 = S[Y + 10];
    const double v10 = S[vb + 10];
    const double y11 = S[Y + 11];
    const double v11 = S[vb + 11];
    const double y12 = S[Y + 12];
    const double v12 = S[vb + 12];
    const double y13 = S[Y + 13];
    const double v13 = S[vb + 13];
    { const double s = -u(12) + u(9) + u(10);
      S[KB + 0] = fma(s, v12, S[KB + 0]);
      const double ks = k(0) * s;
    }
    { const double s = -u(10) - u(3) + u(7);
      S[KB + 1] = fma(s, (y10) * v3 + (y3) * v10, S[KB + 1]);
      const double ks = k(1) * s;
      S[LAM + 3] = fma(ks, v10, S[LAM + 3]);
      S[LAM + 10] = fma(ks, v3, S[LAM + 10]);
    }
    { const double s = fma(2.0, u(3), -u(10) - u(7));
      S[KB + 2] = fma(s, (y10) * v7 + (y7) * v10, S[KB + 2]);
      const double ks = k(2) * s;
      S[LAM + 7] = fma(ks, v10, S[LAM + 7]);
      S[LAM + 10] = fma(ks, v7, S[LAM + 10]);
    }
    { const double s = -u(7) - u(9) + u(12);
      S[KB + 3] = fma(s, (y9) * v7 + (y7) * v9, S[KB + 3]);
      const double ks = k(3) * s;
      S[LAM + 7] = fma(ks, v9, S[LAM + 7]);
      S[LAM + 9] = fma(ks, v7, S[LAM + 9]);
    }
    { const double s = -u(7) - u(12) + u(11);
      S[KB + 4] = fma(s, (y12) * v7 + (y7) * v12, S[KB + 4]);
      const double ks = k(4) * s;
      S[LAM + 7] = fma(ks, v12, S[LAM + 7]);
      S[LAM + 12] = fma(ks, v7, S[LAM + 12]);
    }
    { const double s = fma(2.0, u(12), -u(9) - u(11));
      S[KB + 5] = fma(s, (y11) * v9 + (y9) * v11, S[KB + 5]);
      const double ks = k(5) * s;
      S[LAM + 9] = fma(ks, v11, S[LAM + 9]);
      S[LAM + 11] = fma(ks, v9, S[LAM + 11]);
    }
    { const double s = -u(12) - u(11) + u(13);
      S[KB + 6] = fma(s, (y12) * v11 + (y11) * v12, S[KB + 6]);
      const double ks = k(6) * s;
      S[LAM + 11] = fma(ks, v12, S[LAM + 11]);
      S[LAM + 12] = fma(ks, v11, S[LAM + 12]);
    }
    { const double s = -u(13) + u(12) + u(11);
      S[KB + 7] = fma(s, v13, S[KB + 7]);
      const double ks = k(7) * s;
    }
    { const double s = -u(6) - u(8) + u(11);
      S[KB + 8] = fma(s, (y8) * v6 + (y6) * v8, S[KB + 8]);
      const double ks = k(8) * s;
      S[LAM + 6] = fma(ks, v8, S[LAM + 6]);
      S[LAM + 8] = fma(ks, v6, S[LAM + 8]);
    }
    { const double s = -u(4) + u(5) + u(3);
      S[KB + 9] = fma(s, v4, S[KB + 9]);
      const double ks = k(9) * s;
    }
    { const double s = -u(2) + u(6) + u(9);
      S[KB + 10] = fma(s, v2, S[KB + 10]);
      const double ks = k(10) * s;
    }
    { const double s = -u(8) + u(6) + u(12);
      S[KB + 11] = fma(s, v8, S[KB + 11]);
      const double ks = k(11) * s;
    }
    { const double s = fma(2.0, u(6), -u(5));
      S[KB + 12] = fma(s, v5, S[KB + 12]);
      const double ks = k(12) * s;
    }
  }

  // Adjoint of F_i = f(Y_i): Ybar = J(Y_i)^T Fbar, kbar += m_r(Y_i) (net_r.Fbar).
  // yv(i) supplies Y_i, ybar(j, x) receives Ybar_j.
  template <class SA, class KA, class YA, class OUT>
  __device__ __forceinline__ static void adj_fterm(SA& S, const KA& k, const YA& yv, OUT&& ybar) {
    auto fb = [&](int i) { return S[FBAR + i]; };
    const double y2 = yv(2);
    const double y3 = yv(3);
    const double y4 = yv(4);
    const double y5 = yv(5);
    const double y6 = yv(6);
    const double y7 = yv(7);
    const double y8 = yv(8);
    const double y9 = yv(9);
    const double y10 = yv(10);
    const double y11 = yv(11);
    const double y12 = yv(12);
    const double y13 = yv(13);
    const double s0 = -fb(12) + fb(9) + fb(10);
    S[KB + 0] = fma(s0, y12, S[KB + 0]);
    const double s1 = -fb(10) - fb(3) + fb(7);
    S[KB + 1] = fma(s1, y3 * y10, S[KB + 1]);
    const double s2 = fma(2.0, fb(3), -fb(10) - fb(7));
    S[KB + 2] = fma(s2, y7 * y10, S[KB + 2]);
    const double s3 = -fb(7) - fb(9) + fb(12);
    S[KB + 3] = fma(s3, y7 * y9, S[KB + 3]);
    const double s4 = -fb(7) - fb(12) + fb(11);
    S[KB + 4] = fma(s4, y7 * y12, S[KB + 4]);
    const double s5 = fma(2.0, fb(12), -fb(9) - fb(11));
    S[KB + 5] = fma(s5, y9 * y11, S[KB + 5]);
    const double s6 = -fb(12) - fb(11) + fb(13);
    S[KB + 6] = fma(s6, y11 * y12, S[KB + 6]);
    const double s7 = -fb(13) + fb(12) + fb(11);
    S[KB + 7] = fma(s7, y13, S[KB + 7]);
    const double s8 = -fb(6) - fb(8) + fb(11);
    S[KB + 8] = fma(s8, y6 * y8, S[KB + 8]);
    const double s9 = -fb(4) + fb(5) + fb(3);
    S[KB + 9] = fma(s9, y4, S[KB + 9]);
    const double s10 = -fb(2) + fb(6) + fb(9);
    S[KB + 10] = fma(s10, y2, S[KB + 10]);
    const double s11 = -fb(8) + fb(6) + fb(12);
    S[KB + 11] = fma(s11, y8, S[KB + 11]);
    const double s12 = fma(2.0, fb(6), -fb(5));
    S[KB + 12] = fma(s12, y5, S[KB + 12]);
    ybar(2, k(10) * s10);
    ybar(3, k(1) * s1 * y10);
    ybar(4, k(9) * s9);
    ybar(5, k(12) * s12);
    ybar(6, k(8) * s8 * y8);
    ybar(7, k(2) * s2 * y10 + k(3) * s3 * y9 + k(4) * s4 * y12);
    ybar(8, k(8) * s8 * y6 + k(11) * s11);
    ybar(9, k(3) * s3 * y7 + k(5) * s5 * y11);
    ybar(10, k(1) * s1 * y3 + k(2) * s2 * y7);
    ybar(11, k(5) * s5 * y9 + k(6) * s6 * y12);
    ybar(12, k(0) * s0 + k(4) * s4 * y7 + k(6) * s6 * y11);
    ybar(13, k(7) * s7);
  }

  // Reverse of one accepted step of size h.  Requires the values attempt()
  // left in S for this step (LU, K_i) and y_n in S[Y..].
  template <class SA, class KA>
  __device__ __forceinline__ static void adjoint_step(SA& S, const KA& k, double h) {
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 0 + j] = 1.0 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 14 + j] = 6.1697947043828245 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[KBAR + 28 + j] = -0.42772256543218573 * S[LAM + j];
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 3
    solve_t(S, KBAR + 28);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 28, 95);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 28 + j];
    { const double cc = 4.0759956452537702 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 28 + q], S[KBAR + 0 + q]); }
    { const double cc = 9.20767942983308 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 14 + q] = fma(cc, S[KBAR + 28 + q], S[KBAR + 14 + q]); }
    // stage 2
    solve_t(S, KBAR + 14);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 14, 81);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 14 + j];
    { const double cc = -1.0156171083877703 / h;
      #pragma unroll
      for (int q = 0; q < NV; ++q) S[KBAR + 0 + q] = fma(cc, S[KBAR + 14 + q], S[KBAR + 0 + q]); }
    adj_fterm(S, k, [&](int q) { return S[Y + q] + S[67 + q]; },
              [&](int j, double x) { S[LAM + j] += x; S[KBAR + 0 + j] = fma(1.0, x, S[KBAR + 0 + j]); });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
    // stage 1
    solve_t(S, KBAR + 0);                       // u_i = W^-T Kbar_i
    adj_wterm(S, k, KBAR + 0, 67);       // J(y_n) in W
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] += S[KBAR + 0 + j];
    adj_fterm(S, k, [&](int q) { return S[Y + q]; },
              [&](int j, double x) { S[LAM + j] += x; });
    #pragma unroll
    for (int j = 0; j < NV; ++j) S[FBAR + j] = 0.0;
  }
};

}  // namespace mkpp_saprc99_mini
