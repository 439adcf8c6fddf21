// Generated by gen_hankel.py: float-float pieces of the Hankel evaluator
// for x >= 4 (see hankel_ff.cuh).  Do not edit by hand.
#pragma once
#include "ff.cuh"

namespace bem2d_gpu {

// x in [8, 16): P0, (x/8) Q0, P1, (x/8) Q1 in t = 2 (s - 0.25)/(1 - 0.25) - 1,
// s = (8/x)^2
__host__ __device__ __forceinline__ ff hkff_0_0(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(8.157953886e-15f, t.hi, -4.813773620e-14f), t.hi, 2.977758285e-13f), t.hi, -2.305387652e-12f), t.hi, 2.111152919e-11f), t.hi, -2.393353571e-10f), t.hi, 3.613838340e-09f);
  ff y = ff_add_f(ff_make(-8.149908126e-08f, -2.827701545e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(3.368295438e-06f, 3.358971155e-14f), t, y);
  y = ff_horner_fast(ff_make(-4.000022309e-04f, -1.114199271e-11f), t, y);
  y = ff_horner_fast(ff_make(9.993235469e-01f, 1.750196255e-08f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_0_1(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-2.915657076e-16f, t.hi, 1.367555340e-15f), t.hi, -6.034843357e-15f), t.hi, 3.431652342e-14f), t.hi, -2.162804983e-13f), t.hi, 1.526000246e-12f), t.hi, -1.249619418e-11f), t.hi, 1.235907349e-10f), t.hi, -1.564620877e-09f);
  ff y = ff_add_f(ff_make(2.774588914e-08f, 6.136798172e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(-8.020534210e-07f, 2.723028305e-14f), t, y);
  y = ff_horner_fast(ff_make(5.070442785e-05f, -2.454122517e-13f), t, y);
  y = ff_horner_fast(ff_make(-1.553812250e-02f, 2.658160914e-10f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_0_2(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-8.766389510e-15f, t.hi, 5.199140746e-14f), t.hi, -3.239078385e-13f), t.hi, 2.527921015e-12f), t.hi, -2.339939527e-11f), t.hi, 2.693449908e-10f), t.hi, -4.162371336e-09f);
  ff y = ff_add_f(ff_make(9.764687547e-08f, 6.559651842e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(-4.376802281e-06f, 1.253659042e-13f), t, y);
  y = ff_horner_fast(ff_make(6.711526657e-04f, -1.043188539e-11f), t, y);
  y = ff_horner_fast(ff_make(1.001131177e+00f, 5.686173665e-08f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_0_3(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(3.101923591e-16f, t.hi, -1.459567576e-15f), t.hi, 6.471695094e-15f), t.hi, -3.696431453e-14f), t.hi, 2.342306579e-13f), t.hi, -1.664246865e-12f), t.hi, 1.375393202e-11f), t.hi, -1.377569725e-10f), t.hi, 1.776470859e-09f);
  ff y = ff_add_f(ff_make(-3.244905145e-08f, -8.219780833e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(9.907389540e-07f, -4.501546540e-16f), t, y);
  y = ff_horner_fast(ff_make(-7.148936129e-05f, 1.151341609e-12f), t, y);
  y = ff_horner_fast(ff_make(4.675293341e-02f, -4.784950214e-10f), t, y);
  return y;
}

// x in [16, 64): P0, (x/16) Q0, P1, (x/16) Q1 in t = 2 (s - 0.0625)/(1 - 0.0625) - 1,
// s = (16/x)^2
__host__ __device__ __forceinline__ ff hkff_1_0(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(2.836302529e-16f, t.hi, -3.952587769e-15f), t.hi, 6.944991186e-14f), t.hi, -1.657858204e-12f), t.hi, 5.730775923e-11f), t.hi, -3.231265921e-09f);
  ff y = ff_add_f(ff_make(3.645652384e-07f, -3.611797191e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(-1.279068820e-04f, -3.521601847e-12f), t, y);
  y = ff_horner_fast(ff_make(9.998545647e-01f, 1.131000182e-09f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_1_1(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(1.226322721e-17f, t.hi, -1.268627450e-16f), t.hi, 1.549724916e-15f), t.hi, -2.415473352e-14f), t.hi, 4.898077386e-13f), t.hi, -1.379106551e-11f), t.hi, 5.932979108e-10f);
  ff y = ff_add_f(ff_make(-4.545863774e-08f, -7.347227312e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(8.276492736e-06f, 4.070946393e-14f), t, y);
  y = ff_horner_fast(ff_make(-7.803060580e-03f, -1.183232956e-10f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_1_2(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(-3.039536438e-16f, t.hi, 4.271659151e-15f), t.hi, -7.592448941e-14f), t.hi, 1.841640555e-12f), t.hi, -6.522651169e-11f), t.hi, 3.831822859e-09f);
  ff y = ff_add_f(ff_make(-4.698935356e-07f, 8.975996284e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(2.134964743e-04f, -6.323998616e-12f), t, y);
  y = ff_horner_fast(ff_make(1.000242591e+00f, -1.899915603e-08f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_1_3(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-1.301703855e-17f, t.hi, 1.354391918e-16f), t.hi, -1.667095942e-15f), t.hi, 2.623619671e-14f), t.hi, -5.391522732e-13f), t.hi, 1.547933656e-11f), t.hi, -6.869294578e-10f);
  ff y = ff_add_f(ff_make(5.570204564e-08f, 1.382253082e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(-1.160566444e-05f, -1.586087219e-13f), t, y);
  y = ff_horner_fast(ff_make(2.342427522e-02f, -8.787405803e-10f), t, y);
  return y;
}

// x in [64, inf): P0, (x/64) Q0, P1, (x/64) Q1 in t = 2 (s - 0.0)/(1 - 0.0) - 1,
// s = (64/x)^2
__host__ __device__ __forceinline__ ff hkff_2_0(ff t) {
  const float tail = fmaf(fmaf(1.333961907e-15f, t.hi, -1.036012422e-12f), t.hi, 1.668080452e-09f);
  ff y = ff_add_f(ff_make(-8.579729183e-06f, -3.902570541e-13f), t.hi * tail);
  y = ff_horner_fast(ff_make(9.999914169e-01f, 1.670156458e-09f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_2_1(ff t) {
  const float tail = fmaf(fmaf(fmaf(2.279533475e-19f, t.hi, -8.343479671e-17f), t.hi, 4.876893838e-14f), t.hi, -5.273089257e-11f);
  ff y = ff_add_f(ff_make(1.395927711e-07f, 6.645530819e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(-1.952985302e-03f, -5.282868240e-11f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_2_2(ff t) {
  const float tail = fmaf(fmaf(-1.512234391e-15f, t.hi, 1.224637362e-12f), t.hi, -2.144998179e-09f);
  ff y = ff_add_f(ff_make(1.430082102e-05f, 4.806670063e-14f), t.hi * tail);
  y = ff_horner_fast(ff_make(1.000014305e+00f, -2.147451994e-09f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_2_3(ff t) {
  const float tail = fmaf(fmaf(fmaf(-2.497464547e-19f, t.hi, 9.327624092e-17f), t.hi, -5.628396376e-14f), t.hi, 6.445888961e-11f);
  ff y = ff_add_f(ff_make(-1.954486493e-07f, -4.400672010e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(5.859179422e-03f, 6.457173685e-11f), t, y);
  return y;
}

// x in [4, 8): P0, (x/4) Q0, P1, (x/4) Q1 in t = 2 (s - 0.25)/(1 - 0.25) - 1,
// s = (4/x)^2
__host__ __device__ __forceinline__ ff hkff_3_0(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-9.966476971e-14f, t.hi, 2.834943380e-13f), t.hi, -4.609592330e-13f), t.hi, 1.563911869e-12f), t.hi, -6.037730212e-12f), t.hi, 2.135572448e-11f), t.hi, -7.985621886e-11f), t.hi, 3.236383106e-10f), t.hi, -1.432233110e-09f), t.hi, 7.083329034e-09f);
  ff y = ff_add_f(ff_make(-4.054247782e-08f, -4.227331005e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(2.835932378e-07f, -1.179624246e-14f), t, y);
  y = ff_horner_fast(ff_make(-2.660637392e-06f, -4.541433215e-14f), t, y);
  y = ff_horner_fast(ff_make(4.005517985e-05f, 1.619732235e-12f), t, y);
  y = ff_horner_fast(ff_make(-1.484501641e-03f, 3.700010090e-11f), t, y);
  y = ff_horner_fast(ff_make(9.973993301e-01f, -2.831054680e-08f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_3_1(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-8.603064618e-15f, t.hi, 2.193270861e-14f), t.hi, -1.847712081e-14f), t.hi, 5.969276316e-14f), t.hi, -2.642188497e-13f), t.hi, 7.824213282e-13f), t.hi, -2.333518795e-12f), t.hi, 7.571226632e-12f), t.hi, -2.571285199e-11f), t.hi, 9.176995969e-11f), t.hi, -3.488292433e-10f), t.hi, 1.432085894e-09f), t.hi, -6.473263259e-09f);
  ff y = ff_add_f(ff_make(3.313157393e-08f, -1.652424908e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(-2.004139503e-07f, 6.548905959e-15f), t, y);
  y = ff_horner_fast(ff_make(1.537146659e-06f, 9.179610299e-15f), t, y);
  y = ff_horner_fast(ff_make(-1.698078631e-05f, -4.527189713e-13f), t, y);
  y = ff_horner_fast(ff_make(3.538296151e-04f, 1.055392058e-11f), t, y);
  y = ff_horner_fast(ff_make(-3.060379811e-02f, 4.511467311e-10f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_3_2(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(1.077778478e-13f, t.hi, -3.073842721e-13f), t.hi, 5.035856714e-13f), t.hi, -1.713513012e-12f), t.hi, 6.628552308e-12f), t.hi, -2.355503119e-11f), t.hi, 8.858114936e-11f), t.hi, -3.614105126e-10f), t.hi, 1.612949552e-09f), t.hi, -8.065939916e-09f);
  ff y = ff_add_f(ff_make(4.687875688e-08f, 5.662665657e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(-3.354862770e-07f, -1.096394484e-16f), t, y);
  y = ff_horner_fast(ff_make(3.270190973e-06f, 6.238468130e-14f), t, y);
  y = ff_horner_fast(ff_make(-5.324109952e-05f, -1.221442001e-12f), t, y);
  y = ff_horner_fast(ff_make(2.532773418e-03f, 7.705639946e-12f), t, y);
  y = ff_horner_fast(ff_make(1.004387736e+00f, 4.432021328e-08f), t, y);
  return y;
}
__host__ __device__ __forceinline__ ff hkff_3_3(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(fmaf(-2.355683330e-14f, t.hi, 6.154680308e-14f), t.hi, -6.479468654e-14f), t.hi, 2.083127507e-13f), t.hi, -8.497687146e-13f), t.hi, 2.622495103e-12f), t.hi, -8.282361776e-12f), t.hi, 2.819539567e-11f), t.hi, -1.012866249e-10f), t.hi, 3.872884236e-10f), t.hi, -1.601550559e-09f), t.hi, 7.307455530e-09f);
  ff y = ff_add_f(ff_make(-3.787590330e-08f, -4.528970290e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(2.332946707e-07f, -4.871077686e-15f), t, y);
  y = ff_horner_fast(ff_make(-1.841078415e-06f, 9.906881257e-15f), t, y);
  y = ff_horner_fast(ff_make(2.142969970e-05f, -9.038700235e-13f), t, y);
  y = ff_horner_fast(ff_make(-5.072252243e-04f, -1.697871357e-11f), t, y);
  y = ff_horner_fast(ff_make(9.283403307e-02f, -2.668786969e-09f), t, y);
  return y;
}

// x <= 4: J0 = A0, J1 = x A1, Y0 = (2/pi) ln x J0 + B0,
//         Y1 = (2/pi) ln x J1 - 2/(pi x) + x B1;  t = x^2/8 - 1
__host__ __device__ __forceinline__ ff hkff_4_0(ff t) {
  const float tail = fmaf(fmaf(fmaf(1.529983246e-14f, t.hi, -1.087432336e-12f), t.hi, 6.474430020e-11f), t.hi, -3.177438757e-09f);
  ff y = ff_add_f(ff_make(1.257728002e-07f, 6.118954153e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(-3.910342002e-06f, 2.304720406e-14f), t, y);
  y = ff_horner_fast(ff_make(9.228174167e-05f, -1.769930123e-12f), t, y);
  y = ff_horner_fast(ff_make(-1.578954165e-03f, 2.818224126e-11f), t, y);
  y = ff_horner_fast(ff_make(1.835270040e-02f, 2.126934046e-10f), t, y);
  y = ff_horner_fast(ff_make(-1.310320646e-01f, 1.043430009e-09f), t, y);
  y = ff_horner_fast(ff_make(4.795280695e-01f, 1.265485583e-08f), t, y);
  y = ff_add_fast(ff_make(-5.659599900e-01f, 1.626348123e-08f), ff_mul(t, y));
  y = ff_add_fast(ff_make(-1.965480894e-01f, -5.885435694e-09f), ff_mul(t, y));
  return y;
}
__host__ __device__ __forceinline__ ff hkff_4_1(ff t) {
  const float tail = fmaf(fmaf(fmaf(-4.590114570e-14f, t.hi, 2.990587812e-12f), t.hi, -1.618607470e-10f), t.hi, 7.149236758e-09f);
  ff y = ff_add_f(ff_make(-2.515456003e-07f, -1.224162170e-14f), t.hi * tail);
  y = ff_horner_fast(ff_make(6.843098618e-06f, -1.537591262e-13f), t, y);
  y = ff_horner_fast(ff_make(-1.384226052e-04f, -4.621060912e-12f), t, y);
  y = ff_horner_fast(ff_make(1.973692561e-03f, 1.102912692e-10f), t, y);
  y = ff_horner_fast(ff_make(-1.835270040e-02f, -2.126934046e-10f), t, y);
  y = ff_horner_fast(ff_make(9.827404469e-02f, 2.942717847e-09f), t, y);
  y = ff_horner_fast(ff_make(-2.397640347e-01f, -6.327427915e-09f), t, y);
  y = ff_add_fast(ff_make(1.414899975e-01f, -4.065870307e-09f), ff_mul(t, y));
  return y;
}
__host__ __device__ __forceinline__ ff hkff_4_2(ff t) {
  const float tail = fmaf(fmaf(fmaf(-3.123848023e-14f, t.hi, 2.161122843e-12f), t.hi, -1.248063597e-10f), t.hi, 5.915436141e-09f);
  ff y = ff_add_f(ff_make(-2.248562510e-07f, -7.426550359e-16f), t.hi * tail);
  y = ff_horner_fast(ff_make(6.662166470e-06f, 1.510437410e-15f), t, y);
  y = ff_horner_fast(ff_make(-1.482141961e-04f, -3.824222623e-12f), t, y);
  y = ff_horner_fast(ff_make(2.351704985e-03f, -2.312123062e-11f), t, y);
  y = ff_horner_fast(ff_make(-2.466011606e-02f, 5.956617422e-10f), t, y);
  y = ff_horner_fast(ff_make(1.503964961e-01f, -6.117502505e-09f), t, y);
  y = ff_horner_fast(ff_make(-4.036971033e-01f, -5.002281256e-09f), t, y);
  y = ff_add_fast(ff_make(5.092768744e-02f, 7.692527726e-10f), ff_mul(t, y));
  y = ff_add_fast(ff_make(5.583839417e-01f, -2.265648646e-08f), ff_mul(t, y));
  return y;
}
__host__ __device__ __forceinline__ ff hkff_4_3(ff t) {
  const float tail = fmaf(fmaf(fmaf(fmaf(-1.229939591e-15f, t.hi, 9.248676857e-14f), t.hi, -5.851945664e-12f), t.hi, 3.067759657e-10f), t.hi, -1.305164243e-08f);
  ff y = ff_add_f(ff_make(4.394457278e-07f, 1.166257748e-15f), t.hi * tail);
  y = ff_horner_fast(ff_make(-1.133734986e-05f, 4.390675920e-13f), t, y);
  y = ff_horner_fast(ff_make(2.146563056e-04f, 4.818976381e-12f), t, y);
  y = ff_horner_fast(ff_make(-2.806317061e-03f, 2.627576282e-11f), t, y);
  y = ff_horner_fast(ff_make(2.306634001e-02f, -2.263386423e-10f), t, y);
  y = ff_horner_fast(ff_make(-1.007763892e-01f, -2.230016616e-09f), t, y);
  y = ff_horner_fast(ff_make(1.516679525e-01f, -6.702047806e-09f), t, y);
  y = ff_add_fast(ff_make(8.248634636e-02f, 3.589323505e-09f), ff_mul(t, y));
  return y;
}

}  // namespace bem2d_gpu
