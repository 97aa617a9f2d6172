// Initial fluid state on the device (initialize_fluid, cpp/initialize.cpp:62-83):
// each particle draws positions until it lies outside every colloid, then a
// velocity; the mean velocity is removed afterwards.  Draws are keyed by
// (particle, attempt), so every particle is placed independently and the result
// is the same as drawing them one after another.
#include "kernels.cuh"

namespace bgb {

// style 0: uniform-box velocities (u - 1/2) vscale, as the reference; style 1:
// Maxwell-Boltzmann with standard deviation vscale (Box-Muller).  Writes the raw
// velocity into wx/wy/wz; k_vfinish turns it into a displacement.
__global__ void __launch_bounds__(256) k_init_fluid(const SysF64 S, int style, double vscale, double rmin,
                                                   int max_attempts, InitOut o) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.N) return;
  const int b = (int)((S.ss->step * S.n_sub - 1) & 1);
  const double *Xc = S.X[b];
  const float4 *xs = S.Xf[b];
  const float Lx = (float)S.Lx, Ly = (float)S.Ly, Lz = (float)S.Lz;
  const float rf = (float)rmin + 0.01f;
  double tx = 0, ty = 0, tz = 0;
  bool placed = false;
  for (int a = 0; a < max_attempts && !placed; ++a) {
    uint4 r = draw4(S.key, DOM_INIT_FPOS, 0, (uint32_t)(i + 1), (uint32_t)a, 0);
    // t.random(point(0,0,0), len): x*len - 0
    tx = __dsub_rn(__dmul_rn(u01(r.x), S.dx.L), 0.0);
    ty = __dsub_rn(__dmul_rn(u01(r.y), S.dy.L), 0.0);
    tz = __dsub_rn(__dmul_rn(u01(r.z), S.dz.L), 0.0);
    placed = true;
    float fx = (float)tx, fy = (float)ty, fz = (float)tz;
    for (int j = 0; j < S.Nc && placed; ++j) {
      float4 c = xs[j];
      float dx = fx - c.x, dy = fy - c.y, dz = fz - c.z;
      dx -= Lx * rintf(dx / Lx); dy -= Ly * rintf(dy / Ly); dz -= Lz * rintf(dz / Lz);
      if (dx * dx + dy * dy + dz * dz > rf * rf) continue;
      // the reference's test: sqrt(((t - pos)^2).sum()) < sigma*0.5 with img()
      double ex = ref_img(__dsub_rn(tx, Xc[3 * j]), S.dx), ey = ref_img(__dsub_rn(ty, Xc[3 * j + 1]), S.dy),
             ez = ref_img(__dsub_rn(tz, Xc[3 * j + 2]), S.dz);
      if (__dsqrt_rn(norm2_ref(ex, ey, ez)) < rmin) placed = false;
    }
  }
  if (!placed) atomicOr(&S.ss->err, ERRB_OCCUPANCY);
  const size_t w = (size_t)i * o.stride;
  o.x[w] = tx; o.y[w] = ty; o.z[w] = tz;
  if (o.id) o.id[i] = i;
  if (o.newpos) o.newpos[i] = i;
  uint4 r = draw4(S.key, DOM_INIT_FVEL, 0, (uint32_t)(i + 1), 0, 0);
  double vx, vy, vz;
  if (style == 0) {
    vx = __dmul_rn(__dsub_rn(__dmul_rn(u01(r.x), 1.0), 0.5), vscale);
    vy = __dmul_rn(__dsub_rn(__dmul_rn(u01(r.y), 1.0), 0.5), vscale);
    vz = __dmul_rn(__dsub_rn(__dmul_rn(u01(r.z), 1.0), 0.5), vscale);
  } else {
    double r0 = sqrt(-2.0 * log(u01(r.x))), r1 = sqrt(-2.0 * log(u01(r.z)));
    double s0, c0, s1, c1;
    sincospi(2.0 * u01(r.y), &s0, &c0);
    sincospi(2.0 * u01(r.w), &s1, &c1);
    vx = r0 * c0 * vscale; vy = r0 * s0 * vscale; vz = r1 * c1 * vscale;
  }
  o.vx[w] = vx; o.vy[w] = vy; o.vz[w] = vz;
}

// per-block sums of the raw velocities, fixed order
__global__ void __launch_bounds__(256) k_vsum(const SysF64 S, double *part, InitOut o) {
  __shared__ double sh[3][256];
  double a[3] = {0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.N; i += gridDim.x * blockDim.x) {
    const size_t w = (size_t)i * o.stride;
    a[0] += o.vx[w]; a[1] += o.vy[w]; a[2] += o.vz[w];
  }
  for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] = a[k];
  __syncthreads();
  for (int s = blockDim.x / 2; s > 0; s >>= 1) {
    if ((int)threadIdx.x < s)
      for (int k = 0; k < 3; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    for (int k = 0; k < 3; ++k) part[blockIdx.x * 3 + k] = sh[k][0];
}

// vel = vel - avr_vel, then (scale != 0) the stored displacement w = fl(vel*dt)
__global__ void __launch_bounds__(256) k_vfinish(const SysF64 S, double ax, double ay, double az, InitOut o,
                                                double scale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= S.N) return;
  const size_t w = (size_t)i * o.stride;
  double vx = __dsub_rn(o.vx[w], ax), vy = __dsub_rn(o.vy[w], ay), vz = __dsub_rn(o.vz[w], az);
  if (scale != 0.0) { vx = __dmul_rn(vx, scale); vy = __dmul_rn(vy, scale); vz = __dmul_rn(vz, scale); }
  o.vx[w] = vx; o.vy[w] = vy; o.vz[w] = vz;
}

// AoS xyz triplets (the reference's point arrays, in particle order) <-> the
// device's SoA (in cell order), with the velocity <-> displacement conversion
// w = fl(v*dt), v = w/dt.  scale: 0 copies, otherwise multiplies (to SoA) or
// divides (from SoA) by it.  Upload puts particle i at position i (id[i] = i when
// id is given); download scatters position i back to particle id[i].
__global__ void __launch_bounds__(256) k_aos_to_soa(const double *aos, double *x, double *y, double *z, int *id,
                                                   int *newpos, int n, double scale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = aos[3 * (size_t)i], b = aos[3 * (size_t)i + 1], c = aos[3 * (size_t)i + 2];
  if (scale != 0.0) { a = __dmul_rn(a, scale); b = __dmul_rn(b, scale); c = __dmul_rn(c, scale); }
  x[i] = a; y[i] = b; z[i] = c;
  if (id) id[i] = i;
  if (newpos) newpos[i] = i;
}

__global__ void __launch_bounds__(256) k_soa_to_aos(double *aos, const double *x, const double *y, const double *z,
                                                   const int *id, int n, double scale) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double a = x[i], b = y[i], c = z[i];
  if (scale != 0.0) { a = __ddiv_rn(a, scale); b = __ddiv_rn(b, scale); c = __ddiv_rn(c, scale); }
  const size_t o = 3 * (size_t)id[i];
  aos[o] = a; aos[o + 1] = b; aos[o + 2] = c;
}

}  // namespace bgb
