// Golden-vector driver for the reference's transform builders.
//
// Compiled (host only, g++) against the reference's own
// src/Interpolator/spatialMappers.cuh / spatialMappers.cu by oracle/Makefile
// target `ref`; the binary lands in oracle/_ref/. It prints, for a fixed list
// of parameter sets, the float matrices produced by
// Spatial3DMapper::AffineInit, Spatial2DMapper::AffineInit and
// Spatial3DMapper::GetMyselfInversed (spatialMappers.cuh:637-850, :999-1033,
// :315-433), one case per line:
//   A3 rx ry rz tx ty tz sx sy sz hx hy hz cx cy cz fx fy fz | m0..m15 | inv0..inv15
//   A2 r tx ty sx sy h cx cy fx fy | m0..m8
#include <cstdio>
#include <cstdint>
#include <cmath>

#include "src/Interpolator/spatialMappers.cuh"

static uint64_t s = 0x9E3779B97F4A7C15ull;
static double uni(double lo, double hi) {
  s = s * 6364136223846793005ull + 1442695040888963407ull;
  double u = (double)(s >> 11) * (1.0 / 9007199254740992.0);
  return lo + (hi - lo) * u;
}

int main() {
  for (int k = 0; k < 24; ++k) {
    float3 rot = {(float)uni(-30, 30), (float)uni(-30, 30), (float)uni(-30, 30)};
    float3 tr = {(float)uni(-20, 20), (float)uni(-20, 20), (float)uni(-20, 20)};
    float3 sc = {(float)uni(0.8, 1.2), (float)uni(0.8, 1.2), (float)uni(0.8, 1.2)};
    float3 sh = {(float)uni(-0.2, 0.2), (float)uni(-0.2, 0.2), (float)uni(-0.2, 0.2)};
    float3 c = {(float)uni(-100, 150), (float)uni(-100, 150), (float)uni(-100, 150)};
    float3 f = {(float)uni(-15, 15), (float)uni(-15, 15), (float)uni(-15, 15)};
    if (k == 0) { rot = {0, 0, 0}; tr = {0, 0, 0}; sc = {1, 1, 1}; sh = {0, 0, 0}; f = {0, 0, 0}; }
    Spatial3DMapper m;
    m.Identity();
    m.SetCenter(c);
    m.SetShift(f);
    m.AffineInit(rot, tr, sc, sh);
    float out[16], inv[16];
    m.GetMatrix(out);
    m.GetMyselfInversed(inv);
    printf("A3 %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g |",
           rot.x, rot.y, rot.z, tr.x, tr.y, tr.z, sc.x, sc.y, sc.z, sh.x, sh.y, sh.z, c.x, c.y, c.z,
           f.x, f.y, f.z);
    for (int i = 0; i < 16; ++i) printf(" %.9g", out[i]);
    printf(" |");
    for (int i = 0; i < 16; ++i) printf(" %.9g", inv[i]);
    printf("\n");
  }
  for (int k = 0; k < 24; ++k) {
    float r = (float)uni(-30, 30);
    float2 tr = {(float)uni(-20, 20), (float)uni(-20, 20)};
    float2 sc = {(float)uni(0.8, 1.2), (float)uni(0.8, 1.2)};
    float h = (float)uni(-0.2, 0.2);
    float2 c = {(float)uni(-100, 150), (float)uni(-100, 150)};
    float2 f = {(float)uni(-15, 15), (float)uni(-15, 15)};
    Spatial2DMapper m;
    m.Identity();
    m.SetCenter(c);
    m.SetShift(f);
    m.AffineInit(r, tr, sc, h);
    float out[9];
    m.GetMatrix(out);
    printf("A2 %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g %.9g |", r, tr.x, tr.y, sc.x, sc.y, h,
           c.x, c.y, f.x, f.y);
    for (int i = 0; i < 9; ++i) printf(" %.9g", out[i]);
    printf("\n");
  }
  return 0;
}
