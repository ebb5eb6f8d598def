// k_bonded.cu — FF_Bonded terms on the device so a whole MD step stays on the GPU.
//
// PD src/mmlib/forcefields/ffbonded.cpp:
//   bonds      k (d - l)^2                          :945-1001
//   angles     k (theta - theta0)^2                 :1054-1183
//   dihedrals  sum Vn (1 + cos(n phi + gamma)), or k (phi - gamma)^2 for n <= 0,
//              phi = -atan2(sin, cos) of the (i-a, a-b, b-j) normals  :1270-1470
//   impropers  same law on the improper quartets   :1594-1619
// Bond lengths are formed in FP64; angle and dihedral algebra runs in FP32 on
// FP64 difference vectors.  Forces go to the sorted-slot fixed-point accumulators.
#include "pdgpu_context.cuh"

namespace pdgpu {

struct BondedView {
  const int* slot_of;          // [natom] sorted slot of each atom
  const int* atom_sys;
  const double* pos;
  long long* facc;
  long long* eacc;
  unsigned* status;
  int nbond, nangle, ntors, nimpr;
  const int *bidx, *aidx, *tidx, *iidx;
  const double *bpar, *apar, *tpar, *ipar;   // kcal/mol units
};

__device__ __forceinline__ void add_force(const BondedView& b, int atom, float fx, float fy, float fz) {
  int s = b.slot_of[atom];
  fix_range(b.status, fabsf(fx) + fabsf(fy) + fabsf(fz));
  atomic_add_ll(&b.facc[3 * s], fx32(fx));
  atomic_add_ll(&b.facc[3 * s + 1], fx32(fy));
  atomic_add_ll(&b.facc[3 * s + 2], fx32(fz));
}

__device__ __forceinline__ float3 dvec(const double* pos, int a, int b) {
  return make_float3((float)(pos[3 * a] - pos[3 * b]), (float)(pos[3 * a + 1] - pos[3 * b + 1]),
                     (float)(pos[3 * a + 2] - pos[3 * b + 2]));
}
__device__ __forceinline__ float3 cross(float3 a, float3 b) {
  return make_float3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
__device__ __forceinline__ float dot(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// PD's dihedral energy in FP64 (energy evaluations only)
__device__ double dihedral_energy_d(const BondedView& b, const int* idx, const double* par) {
  int ti = idx[0], ta = idx[1], tb = idx[2], tj = idx[3], terms = idx[4];
  double v1[3], v2[3], v3[3];
  for (int c = 0; c < 3; c++) {
    v1[c] = b.pos[3 * ti + c] - b.pos[3 * ta + c];
    v2[c] = b.pos[3 * ta + c] - b.pos[3 * tb + c];
    v3[c] = b.pos[3 * tb + c] - b.pos[3 * tj + c];
  }
  double n1[3] = {v1[1] * v2[2] - v1[2] * v2[1], v1[2] * v2[0] - v1[0] * v2[2], v1[0] * v2[1] - v1[1] * v2[0]};
  double n2[3] = {v2[1] * v3[2] - v2[2] * v3[1], v2[2] * v3[0] - v2[0] * v3[2], v2[0] * v3[1] - v2[1] * v3[0]};
  double n3[3] = {v2[1] * n1[2] - v2[2] * n1[1], v2[2] * n1[0] - v2[0] * n1[2], v2[0] * n1[1] - v2[1] * n1[0]};
  double m1 = sqrt(n1[0] * n1[0] + n1[1] * n1[1] + n1[2] * n1[2]);
  double m2 = sqrt(n2[0] * n2[0] + n2[1] * n2[1] + n2[2] * n2[2]);
  double m3 = sqrt(n3[0] * n3[0] + n3[1] * n3[1] + n3[2] * n3[2]);
  double cphi = (n1[0] * n2[0] + n1[1] * n2[1] + n1[2] * n2[2]) / (m1 * m2);
  double sphi = (n3[0] * n2[0] + n3[1] * n2[1] + n3[2] * n2[2]) / (m3 * m2);
  double phi = -atan2(sphi, cphi);
  double E = 0;
  for (int t = 0; t < terms; t++) {
    double k = par[3 * t], n = par[3 * t + 1], g = par[3 * t + 2];
    if (n > 0) {
      E += k * (1.0 + cos(n * phi + g));
    } else {
      double diff = phi - g;
      if (diff < -3.14159265358979323846) diff += 2 * 3.14159265358979323846;
      else if (diff > 3.14159265358979323846) diff -= 2 * 3.14159265358979323846;
      E += k * diff * diff;
    }
  }
  return E;
}

__device__ float dihedral(const BondedView& b, const int* idx, const double* par) {
  int ti = idx[0], ta = idx[1], tb = idx[2], tj = idx[3], terms = idx[4];
  float3 v1 = dvec(b.pos, ti, ta), v2 = dvec(b.pos, ta, tb), v3 = dvec(b.pos, tb, tj);
  float3 n1 = cross(v1, v2), n2 = cross(v2, v3), n3 = cross(v2, n1);
  float m1 = sqrtf(dot(n1, n1)), m2 = sqrtf(dot(n2, n2)), m3 = sqrtf(dot(n3, n3));
  float cphi = dot(n1, n2) / (m1 * m2);
  float sphi = dot(n3, n2) / (m3 * m2);
  float phi = -atan2f(sphi, cphi);
  float E = 0.f, dE = 0.f;
  for (int t = 0; t < terms; t++) {
    float k = (float)par[3 * t], n = (float)par[3 * t + 1], g = (float)par[3 * t + 2];
    if (n > 0.f) {
      float sa, ca;
      sincosf(n * phi + g, &sa, &ca);
      E += k * (1.f + ca);
      dE += -n * k * sa;
    } else {
      float diff = phi - g;
      if (diff < -3.14159265358979f) diff += 6.28318530717959f;
      else if (diff > 3.14159265358979f) diff -= 6.28318530717959f;
      E += k * diff * diff;
      dE += 2.f * k * diff;
    }
  }
  // analytic gradient (F = i-a, G = a-b, H = j-b; Blondel & Karplus 1996)
  float3 F = v1, G = v2, H = make_float3(-v3.x, -v3.y, -v3.z);
  float3 A = cross(F, G), B = cross(H, G);
  float A2 = dot(A, A), B2 = dot(B, B), Gm = sqrtf(dot(G, G));
  float FG = dot(F, G), HG = dot(H, G);
  float s = -dE;
  float ci = -Gm / A2, cj = Gm / B2, ca1 = FG / (A2 * Gm), cb1 = HG / (B2 * Gm);
  float3 gi = make_float3(ci * A.x, ci * A.y, ci * A.z);
  float3 gj = make_float3(cj * B.x, cj * B.y, cj * B.z);
  float3 ga = make_float3(-gi.x + ca1 * A.x - cb1 * B.x, -gi.y + ca1 * A.y - cb1 * B.y, -gi.z + ca1 * A.z - cb1 * B.z);
  float3 gb = make_float3(-gj.x - ca1 * A.x + cb1 * B.x, -gj.y - ca1 * A.y + cb1 * B.y, -gj.z - ca1 * A.z + cb1 * B.z);
  add_force(b, ti, s * gi.x, s * gi.y, s * gi.z);
  add_force(b, ta, s * ga.x, s * ga.y, s * ga.z);
  add_force(b, tb, s * gb.x, s * gb.y, s * gb.z);
  add_force(b, tj, s * gj.x, s * gj.y, s * gj.z);
  return E;
}

template <bool ENERGY>
__global__ void k_bonded(BondedView b) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int total = b.nbond + b.nangle + b.ntors + b.nimpr;
  if (t >= total) return;
  double E = 0.0;
  int slot, sys;
  if (t < b.nbond) {
    int i = b.bidx[2 * t], j = b.bidx[2 * t + 1];
    double l = b.bpar[2 * t], k = b.bpar[2 * t + 1];
    double vx = b.pos[3 * i] - b.pos[3 * j], vy = b.pos[3 * i + 1] - b.pos[3 * j + 1], vz = b.pos[3 * i + 2] - b.pos[3 * j + 2];
    double d = sqrt(vx * vx + vy * vy + vz * vz);
    double dl = d - l;
    E = k * dl * dl;
    float f = (float)(2.0 * k * dl / d);
    add_force(b, i, -f * (float)vx, -f * (float)vy, -f * (float)vz);
    add_force(b, j, f * (float)vx, f * (float)vy, f * (float)vz);
    slot = E_BOND;
    sys = b.atom_sys[i];
  } else if (t < b.nbond + b.nangle) {
    int q = t - b.nbond;
    int i = b.aidx[3 * q], a = b.aidx[3 * q + 1], j = b.aidx[3 * q + 2];
    float theta0 = (float)b.apar[2 * q], k = (float)b.apar[2 * q + 1];
    sys = b.atom_sys[i];
    slot = E_ANGLE;
    if (k != 0.f) {
      float3 u = dvec(b.pos, i, a), w = dvec(b.pos, j, a);
      float lu = sqrtf(dot(u, u)), lw = sqrtf(dot(w, w));
      float ct = dot(u, w) / (lu * lw);
      ct = fminf(1.f, fmaxf(-1.f, ct));
      float th = acosf(ct);
      float st = sinf(th);
      if (ENERGY) {
        double ud[3], wd[3];
        for (int c = 0; c < 3; c++) {
          ud[c] = b.pos[3 * i + c] - b.pos[3 * a + c];
          wd[c] = b.pos[3 * j + c] - b.pos[3 * a + c];
        }
        double cd = (ud[0] * wd[0] + ud[1] * wd[1] + ud[2] * wd[2]) /
                    sqrt((ud[0] * ud[0] + ud[1] * ud[1] + ud[2] * ud[2]) * (wd[0] * wd[0] + wd[1] * wd[1] + wd[2] * wd[2]));
        double thd = acos(fmin(1.0, fmax(-1.0, cd)));
        E = b.apar[2 * q + 1] * (thd - b.apar[2 * q]) * (thd - b.apar[2 * q]);
      }
      float dEdth = 2.f * k * (th - theta0);
      float3 gi, gj;
      gi.x = (ct * u.x / lu - w.x / lw) / (lu * st);
      gi.y = (ct * u.y / lu - w.y / lw) / (lu * st);
      gi.z = (ct * u.z / lu - w.z / lw) / (lu * st);
      gj.x = (ct * w.x / lw - u.x / lu) / (lw * st);
      gj.y = (ct * w.y / lw - u.y / lu) / (lw * st);
      gj.z = (ct * w.z / lw - u.z / lu) / (lw * st);
      add_force(b, i, -dEdth * gi.x, -dEdth * gi.y, -dEdth * gi.z);
      add_force(b, j, -dEdth * gj.x, -dEdth * gj.y, -dEdth * gj.z);
      add_force(b, a, dEdth * (gi.x + gj.x), dEdth * (gi.y + gj.y), dEdth * (gi.z + gj.z));
    }
  } else if (t < b.nbond + b.nangle + b.ntors) {
    int q = t - b.nbond - b.nangle;
    dihedral(b, b.tidx + 5 * q, b.tpar + 12 * q);
    if (ENERGY) E = dihedral_energy_d(b, b.tidx + 5 * q, b.tpar + 12 * q);
    slot = E_TORS;
    sys = b.atom_sys[b.tidx[5 * q]];
  } else {
    int q = t - b.nbond - b.nangle - b.ntors;
    dihedral(b, b.iidx + 5 * q, b.ipar + 12 * q);
    if (ENERGY) E = dihedral_energy_d(b, b.iidx + 5 * q, b.ipar + 12 * q);
    slot = E_IMPR;
    sys = b.atom_sys[b.iidx[5 * q]];
  }
  if (ENERGY) atomic_add_ll(&b.eacc[(size_t)sys * E_NSLOTS + slot], fix_energy_d(E));
}

int launch_bonded(Context& c, bool energy) {
  c.kernel_launches += ((c.nbond + c.nangle + c.ntors + c.nimpr) > 0 ? 1 : 0);
  BondedView b;
  b.slot_of = c.d_slot_of.p;
  b.atom_sys = c.d_atom_sys.p;
  b.pos = c.d_pos.p;
  b.facc = c.d_facc.p;
  b.status = c.d_status.p;
  b.eacc = c.d_eacc.p;
  b.nbond = c.nbond; b.nangle = c.nangle; b.ntors = c.ntors; b.nimpr = c.nimpr;
  b.bidx = c.d_bidx.p; b.aidx = c.d_aidx.p; b.tidx = c.d_tidx.p; b.iidx = c.d_iidx.p;
  b.bpar = c.d_bpar.p; b.apar = c.d_apar.p; b.tpar = c.d_tpar.p; b.ipar = c.d_ipar.p;
  int total = c.nbond + c.nangle + c.ntors + c.nimpr;
  if (total == 0) return PDGPU_OK;
  if (energy) k_bonded<true><<<(total + 255) / 256, 256, 0, c.stream>>>(b);
  else k_bonded<false><<<(total + 255) / 256, 256, 0, c.stream>>>(b);
  return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_ERR_CUDA;
}

}  // namespace pdgpu
