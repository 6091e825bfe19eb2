// Element residual / Jacobian assembly of the shallow-water Newton system.
//
// Restates EQS_UVS2D::Region (CoefsUVS2D.cpp:365-1182), EQS_UVS2D::Bound
// (CoefsUVS2D.cpp:71-360), EQS::Rotate2D (Rotate.cpp:42-107) and the scatter of
// CRSMAT::AssembleEqs_im (Assemble.cpp:195-343) for constant eddy viscosity and
// no dispersion (the Reynolds-stress and dispersion terms are zero then).
//
// GPU layout, two phases.  k_element: one warp per group of four six-node
// triangles; one lane per (triangle, Gauss point) evaluates the Jacobian
// transform, interpolated state, residual integrands and the scalar
// coefficients of the nine Jacobian blocks; all lanes then expand the
// per-Gauss-point trial vectors and accumulate each 15x15 element matrix,
// staged in shared memory for the boundary rotation and the inlet rows, and
// store it by the element's position in the assembly order (elements grouped
// by colour, no two elements of a colour sharing a node).  k_asm_gather: one
// thread per CRS value and per residual row sums its contributions in that
// order -- the sums the colour-by-colour scatter forms, with every value
// written once and no atomics.  The residual is always computed in FP64; the
// Jacobian in FP64 (plain and reference precision) or FP32 (mixed).

#include "rg_internal.cuh"

#include <algorithm>

namespace {

// ---- shape functions at the seven Gauss points of degree 5 (Cowper 1973),
// P1 and P2 triangle, and the three-point line rule (Shape.cpp:308-322,
// Triangle.cpp:201-400, Line.cpp:115-152) -- filled by init_shape_tables()
struct ShapeTables {
  double w[7];
  double m[7][3];
  double n[7][6], dnx[7][6], dny[7][6];
  double lw[3], lm[3][2], ln[3][3], ldn[3][3];
};
__constant__ ShapeTables cS;
// the P2 / P1 values again in FP32, for the FP32 Jacobian (same roundings as a cast)
struct ShapeTablesF {
  float n[7][6], m[7][3];
};
__constant__ ShapeTablesF cSf;
template <class KT>
__device__ __forceinline__ KT shape_n(int g, int k) {
  if constexpr (sizeof(KT) == 4) return cSf.n[g][k]; else return cS.n[g][k];
}
template <class KT>
__device__ __forceinline__ KT shape_m(int g, int k) {
  if constexpr (sizeof(KT) == 4) return cSf.m[g][k]; else return cS.m[g][k];
}

ShapeTables make_tables() {
  ShapeTables t;
  const double loc[7][2] = {{1.0 / 3.0, 1.0 / 3.0},
                            {0.0597158717897698, 0.470142064105115},
                            {0.470142064105115, 0.0597158717897698},
                            {0.470142064105115, 0.470142064105115},
                            {0.797426985353087, 0.101286507323456},
                            {0.101286507323456, 0.797426985353087},
                            {0.101286507323456, 0.101286507323456}};
  const double w[7] = {0.1125, 0.0661970763942531, 0.0661970763942531, 0.0661970763942531,
                       0.0629695902724136, 0.0629695902724136, 0.0629695902724136};
  for (int g = 0; g < 7; g++) {
    double L[3] = {1.0 - loc[g][0] - loc[g][1], loc[g][0], loc[g][1]};
    double dLx[3] = {-1.0, 1.0, 0.0}, dLy[3] = {-1.0, 0.0, 1.0};
    t.w[g] = w[g];
    for (int i = 0; i < 3; i++) {
      t.m[g][i] = L[i];
      t.n[g][i] = (2.0 * L[i] - 1.0) * L[i];
      t.dnx[g][i] = (4.0 * L[i] - 1.0) * dLx[i];
      t.dny[g][i] = (4.0 * L[i] - 1.0) * dLy[i];
    }
    for (int k = 3; k < 6; k++) {
      int i = k % 3, j = (k + 1) % 3;
      t.n[g][k] = 4.0 * L[i] * L[j];
      t.dnx[g][k] = 4.0 * (dLx[i] * L[j] + L[i] * dLx[j]);
      t.dny[g][k] = 4.0 * (dLy[i] * L[j] + L[i] * dLy[j]);
    }
  }
  for (int g = 0; g < 3; g++) {
    double x = (g == 0) ? -sqrt(0.6) : (g == 1 ? 0.0 : sqrt(0.6));
    t.lw[g] = (g == 1) ? 8.0 / 9.0 : 5.0 / 9.0;
    t.lm[g][0] = (1.0 - x) / 2.0;
    t.lm[g][1] = (1.0 + x) / 2.0;
    t.ln[g][0] = x * (x - 1.0) / 2.0;
    t.ln[g][1] = x * (x + 1.0) / 2.0;
    t.ln[g][2] = 1.0 - x * x;
    t.ldn[g][0] = x - 0.5;
    t.ldn[g][1] = x + 0.5;
    t.ldn[g][2] = -2.0 * x;
  }
  return t;
}

struct AsmArgs {
  const double *x, *y, *z, *U, *V, *S, *dUdt, *dVdt, *dSdt, *cf, *cfw;
  const int *nflag, *bckind;
  const double *rot, *niox, *nioy, *bcU, *bcS;
  const int *enodes, *eflag;
  const double* evt;
  const int* elems;  // the assembly order: element ids grouped by colour
  const int* reg;    // positions in elems of the region triangles
  int count;
  const int* bnd;    // positions in elems of the boundary line elements
  int bcount;
  double g, hmin, vk, rUV, rH;
  const double* geo;   // k_geometry output, per element of the list
  int jac_friction;    // add the depth derivative of the friction coefficient to the U-H / V-H blocks
};

// block-coefficient slots per Gauss point
enum {
  C_W, C_H, C_U, C_V,
  C_UU0, C_UUX, C_UUY, C_UUXX, C_UUYY,   // U-derivative of x-momentum
  C_UV0, C_UVYX,                         // V-derivative of x-momentum
  C_UH0, C_UHX, C_UHY,                   // H-derivative of x-momentum
  C_VU0, C_VUXY,                         // U-derivative of y-momentum
  C_VV0, C_VVX, C_VVY, C_VVXX, C_VVYY,   // V-derivative of y-momentum
  C_VH0, C_VHX, C_VHY,                   // H-derivative of y-momentum
  C_SU0, C_SUX,                          // U-derivative of continuity
  C_SV0, C_SVY,                          // V-derivative of continuity
  C_SH0, C_SHX, C_SHY,                   // H-derivative of continuity
  C_UF, C_VF,                            // friction force per unit cf (w |U| U, w |U| V)
  C_N
};

// Mesh geometry of the region triangles in the assembly lists, per Gauss
// point: the integration weight detJ*w and the x/y derivatives of the P2 and
// P1 shape functions (Jacobian transform of CoefsUVS2D.cpp:365-460).  It
// depends on the node coordinates only, so it is computed once per element
// list instead of once per Newton iteration; the arithmetic is the element
// kernel's own.
constexpr int GEO_PER_GP = 19;                  // w, dndx[6], dndy[6], dmdx[3], dmdy[3]
constexpr int GEO_PER_ELEM = 7 * GEO_PER_GP;

template <class KT>
__global__ void k_geometry(AsmArgs a, double* __restrict__ geo) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < a.count * 7; t += gridDim.x * blockDim.x) {
    const int g = t % 7;
    const int e = a.elems[a.reg[t / 7]];
    const int* nd = a.enodes + 6 * e;
    double* o = geo + (size_t)e * GEO_PER_ELEM + g * GEO_PER_GP;
    double x[6], y[6];
    x[0] = 0.0;
    y[0] = 0.0;
    for (int i = 1; i < 6; i++) {
      x[i] = a.x[nd[i]] - a.x[nd[0]];
      y[i] = a.y[nd[i]] - a.y[nd[0]];
    }
    double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
    for (int k = 0; k < 6; k++) {
      j00 += cS.dnx[g][k] * x[k];
      j01 += cS.dnx[g][k] * y[k];
      j10 += cS.dny[g][k] * x[k];
      j11 += cS.dny[g][k] * y[k];
    }
    double detj = j00 * j11 - j01 * j10;
    double t00, t01, t10, t11;
    if constexpr (sizeof(KT) == 4) {   // mixed: one FP64 division instead of four
      const double idet = 1.0 / detj;
      t00 = j11 * idet, t01 = -j01 * idet, t10 = -j10 * idet, t11 = j00 * idet;
    } else {
      t00 = j11 / detj, t01 = -j01 / detj, t10 = -j10 / detj, t11 = j00 / detj;
    }
    o[0] = detj * cS.w[g];
    double dndx[6], dndy[6], dmdx[3], dmdy[3];
    for (int j = 0; j < 6; j++) {
      dndx[j] = t00 * cS.dnx[g][j] + t01 * cS.dny[g][j];
      dndy[j] = t10 * cS.dnx[g][j] + t11 * cS.dny[g][j];
      o[1 + j] = dndx[j];
      o[7 + j] = dndy[j];
    }
    const double dLx[3] = {-1.0, 1.0, 0.0}, dLy[3] = {-1.0, 0.0, 1.0};
    for (int j = 0; j < 3; j++) {
      dmdx[j] = t00 * dLx[j] + t01 * dLy[j];
      dmdy[j] = t10 * dLx[j] + t11 * dLy[j];
      o[13 + j] = dmdx[j];
      o[16 + j] = dmdy[j];
    }
  }
}

// Jacobian block coefficients of one Gauss point (CoefsUVS2D.cpp:749-1059),
// evaluated in R: FP64 for the FP64 Jacobian, FP32 for the FP32 one
template <class R, class KT>
__device__ __forceinline__ void block_coefs(KT* c, R w, R H, R U, R V, R dUdx, R dUdy, R dVdx, R dVdy, R dUdt,
                                            R dVdt, R dHdx, R dHdy, R dadx, R dady, R cf, R Ures, R iUres, R vt,
                                            R gr, R rUV, R rH) {
  c[C_W] = (KT)w;
  c[C_H] = (KT)H;
  c[C_U] = (KT)U;
  c[C_V] = (KT)V;
  c[C_UU0] = (KT)(w * H * rUV + w * H * dUdx + w * cf * (iUres * U * U + Ures));
  c[C_UUX] = (KT)(w * H * U);
  c[C_UUY] = (KT)(w * H * V);
  c[C_UUXX] = (KT)(w * H * vt * (R)2.0);
  c[C_UUYY] = (KT)(w * H * vt);
  c[C_UV0] = (KT)(w * H * dUdy + w * cf * iUres * U * V);
  c[C_UVYX] = (KT)(w * H * vt);
  c[C_UH0] = (KT)(w * dUdt + w * (U * dUdx + V * dUdy) + w * gr * dadx);
  c[C_UHX] = (KT)(w * vt * (dUdx + dUdx) - w * gr * H);
  c[C_UHY] = (KT)(w * vt * (dUdy + dVdx));
  c[C_VU0] = (KT)(w * H * dVdx + w * cf * iUres * U * V);
  c[C_VUXY] = (KT)(w * H * vt);
  c[C_VV0] = (KT)(w * H * rUV + w * H * dVdy + w * cf * (iUres * V * V + Ures));
  c[C_VVX] = (KT)(w * H * U);
  c[C_VVY] = (KT)(w * H * V);
  c[C_VVXX] = (KT)(w * H * vt);
  c[C_VVYY] = (KT)(w * H * vt * (R)2.0);
  c[C_VH0] = (KT)(w * dVdt + w * (U * dVdx + V * dVdy) + w * gr * dady);
  c[C_VHX] = (KT)(w * vt * (dVdx + dUdy));
  c[C_VHY] = (KT)(w * vt * (dVdy + dVdy) - w * gr * H);
  c[C_SU0] = (KT)(w * dHdx);
  c[C_SUX] = (KT)(w * H);
  c[C_SV0] = (KT)(w * dHdy);
  c[C_SVY] = (KT)(w * H);
  c[C_SH0] = (KT)(w * rH + w * (dUdx + dVdy));
  c[C_SHX] = (KT)(w * U);
  c[C_SHY] = (KT)(w * V);
  c[C_UF] = (KT)(w * Ures * U);
  c[C_VF] = (KT)(w * Ures * V);
}

template <class KT>
struct GpData {              // node data and Gauss-point results of one element
  double nd[10][6];          // per node: U V dUdt dVdt S z dSdt cf x y
  KT dcf[3];                 // corner depth derivatives of cf (0 unless jac_friction)
  double dndx[7][6], dndy[7][6], dmdx[7][3], dmdy[7][3];
  double res[7][7];          // per GP: ffU fxU fyU ffV fxV fyV fC (already times weight)
  KT coef[7][C_N];
  KT kdndx[7][6], kdndy[7][6], kdmdx[7][3], kdmdy[7][3];   // the derivatives in the Jacobian's type
};

template <class KT, int EPW>
struct WarpSmem {
  GpData<KT> el[EPW];
  KT T[7][9][3][6];          // trial vectors per GP: block (rowvar*3+colvar), {t, tx, ty}, k
  KT K[RG_EQ][RG_KSTRIDE];   // element matrix
  double Kb[9][9];           // boundary-line element matrix
  double f[RG_EQ];
  double area;
};

// Phase 1 of the assembly: every element matrix and residual of the model in
// one launch, stored by the element's position p in the assembly order
// (EK[p][r*15+c], EF[p][r]).  Work items [0, nregw) are groups of EPW region
// triangles: their node loads and Gauss-point evaluations run side by side
// (lane = element * 7 + Gauss point), which keeps 7*EPW lanes of the FP64
// pipe busy instead of 7; matrix expansion, rotation and inlet rows then run
// element by element with all lanes.  Work items from nregw on are boundary
// line elements, one per warp: lane 0 integrates, all lanes store.
template <class KT, int WARPS, int EPW>
__global__ void __launch_bounds__(WARPS * 32, 6) k_element(AsmArgs a, KT* __restrict__ EK, double* __restrict__ EF) {
  __shared__ WarpSmem<KT, EPW> smem[WARPS];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  WarpSmem<KT, EPW>& s = smem[wib];
  const int nwarps = gridDim.x * WARPS;
  const int nregw = (a.count + EPW - 1) / EPW;

  for (int wi = blockIdx.x * WARPS + wib; wi < nregw + a.bcount; wi += nwarps) {
    if (wi >= nregw) {
      const int p = a.bnd[wi - nregw];
      const int e = a.elems[p];
      if (lane == 0) {
        // three-node boundary line (CoefsUVS2D.cpp:71-360): rows U0..2 (0-2), V0..2
        // (3-5), S at the corners (6-7); stored in the 15x15 slot block at [r][c], r, c < 9
        const int* nd = a.enodes + 6 * e;
        double(&K)[9][9] = s.Kb;
        double* f = s.f;
        for (int i = 0; i < 9; i++) {
          f[i] = 0.0;
          for (int j = 0; j < 9; j++) K[i][j] = 0.0;
        }
        const int fl = a.eflag[e];
        const int solid = !(!(a.bckind[nd[2]] & RG_B_LOGLAW) || (fl & RG_E_INLET) || (fl & RG_E_OUTLET) ||
                            (fl & RG_E_OPENBND));
        const int outlet = (a.bckind[nd[2]] & RG_B_OUTLET) != 0;
        const double gr = a.g;
        for (int g = 0; g < 3; g++) {
          const double* m = cS.lm[g];
          const double* n = cS.ln[g];
          const double* dn = cS.ldn[g];
          double H0, H1;
          if (outlet) {
            H0 = a.bcS[nd[0]] - a.z[nd[0]];
            H1 = a.bcS[nd[1]] - a.z[nd[1]];
          } else {
            H0 = a.S[nd[0]] - a.z[nd[0]];
            H1 = a.S[nd[1]] - a.z[nd[1]];
          }
          if (H0 <= 0.0) H0 = a.hmin;
          if (H1 <= 0.0) H1 = a.hmin;
          const double H = m[0] * H0 + m[1] * H1;
          const double nx = dn[0] * a.y[nd[0]] + dn[1] * a.y[nd[1]] + dn[2] * a.y[nd[2]];
          const double ny = -dn[0] * a.x[nd[0]] - dn[1] * a.x[nd[1]] - dn[2] * a.x[nd[2]];
          const double len = sqrt(nx * nx + ny * ny);
          const double weight = cS.lw[g];
          double U = 0, V = 0, Ures = 0, cf = 0;
          if (solid) {
            U = n[0] * a.U[nd[0]] + n[1] * a.U[nd[1]] + n[2] * a.U[nd[2]];
            V = n[0] * a.V[nd[0]] + n[1] * a.V[nd[1]] + n[2] * a.V[nd[2]];
            Ures = sqrt(U * U + V * V);
            cf = m[0] * a.cfw[nd[0]] + m[1] * a.cfw[nd[1]];
          }
          double fU = weight * H * (gr * H / 2.0 * nx);
          double fV = weight * H * (gr * H / 2.0 * ny);
          if (solid) {
            fU += weight * len * H * cf * U * Ures;
            fV += weight * len * H * cf * V * Ures;
          }
          for (int i = 0; i < 3; i++) {
            f[i] -= n[i] * fU;
            f[3 + i] -= n[i] * fV;
          }
          double dUU = 0, dUV = 0, dUH = 0, dVU = 0, dVV = 0, dVH = 0;
          if (!outlet) {
            dUH += weight * (gr * H * nx);
            dVH += weight * (gr * H * ny);
          }
          if (solid) {
            dUH += weight * len * cf * U * Ures;
            dVH += weight * len * cf * V * Ures;
            double iUres = (Ures > 1.0e-8) ? 1.0 / Ures : 0.0;
            dUU += weight * len * cf * H * (U * U * iUres + Ures);
            dUV += weight * len * cf * H * (U * V * iUres);
            dVU += weight * len * cf * H * (U * V * iUres);
            dVV += weight * len * cf * H * (V * V * iUres + Ures);
          }
          for (int i = 0; i < 3; i++) {
            for (int k = 0; k < 3; k++) {
              K[i][k] += n[i] * dUU * n[k];
              K[i][3 + k] += n[i] * dUV * n[k];
              K[3 + i][k] += n[i] * dVU * n[k];
              K[3 + i][3 + k] += n[i] * dVV * n[k];
            }
            for (int k = 0; k < 2; k++) {
              K[i][6 + k] += n[i] * dUH * m[k];
              K[3 + i][6 + k] += n[i] * dVH * m[k];
            }
          }
        }
        for (int i = 0; i < 3; i++) {
          const int n = nd[i];
          if (!(a.nflag[n] & RG_N_ROTAT)) continue;
          const double r00 = a.rot[4 * n], r01 = a.rot[4 * n + 1], r10 = a.rot[4 * n + 2], r11 = a.rot[4 * n + 3];
          if (fabs(r00 * r11 - r01 * r10) < 1.0e-12) continue;
          const int j = 3 + i;
          for (int k = 0; k < 9; k++) {
            double tmp = K[k][i] * r00 + K[k][j] * r10;
            K[k][j] = K[k][i] * r01 + K[k][j] * r11;
            K[k][i] = tmp;
          }
          for (int k = 0; k < 9; k++) {
            double tmp = r00 * K[i][k] + r10 * K[j][k];
            K[j][k] = r01 * K[i][k] + r11 * K[j][k];
            K[i][k] = tmp;
          }
          double tmp = r00 * f[i] + r10 * f[j];
          f[j] = r01 * f[i] + r11 * f[j];
          f[i] = tmp;
        }
        for (int i = 0; i < 3; i++) {
          if (a.bckind[nd[i]] & RG_B_INLET) {
            for (int j = 0; j < 9; j++) K[i][j] = 0.0;
            f[i] = 0.0;
          }
        }
      }
      __syncwarp();
      KT* ek = EK + (size_t)p * (RG_EQ * RG_EQ);
      for (int idx = lane; idx < 81; idx += 32) {
        const int r = idx / 9, c = idx % 9;
        ek[r * RG_EQ + c] = (KT)s.Kb[r][c];
      }
      if (lane < 9) EF[(size_t)p * RG_EQ + lane] = s.f[lane];
      __syncwarp();
      continue;
    }
    const int base = wi * EPW;
    const int nel = min(EPW, a.count - base);

    // 1. node data, one lane per (element, node)
    if (lane < 6 * nel) {
      GpData<KT>& d = s.el[lane / 6];
      const int k = a.enodes[6 * a.elems[a.reg[base + lane / 6]] + lane % 6];
      const int i = lane % 6;
      d.nd[0][i] = a.U[k];
      d.nd[1][i] = a.V[k];
      d.nd[2][i] = a.dUdt[k];
      d.nd[3][i] = a.dVdt[k];
      d.nd[4][i] = a.S[k];
      d.nd[5][i] = a.z[k];
      d.nd[6][i] = a.dSdt[k];
      d.nd[7][i] = a.cf[k];
      d.nd[8][i] = a.x[k];
      d.nd[9][i] = a.y[k];
      if (i < 3) {
        // d cf_k / d h_k of cf_k = C_k / max(h_k, hmin)^0.333333 (k_friction)
        const double h = d.nd[4][i] - d.nd[5][i];
        d.dcf[i] = (a.jac_friction && h > a.hmin) ? (KT)(-0.333333 * d.nd[7][i] / h) : (KT)0;
      }
    }
    __syncwarp();

    // 2. Gauss-point quantities, one lane per (element, Gauss point)
    if (lane < 7 * nel) {
      const int g = lane % 7;
      GpData<KT>& d = s.el[lane / 7];
      const int e = a.elems[a.reg[base + lane / 7]];
      // mesh geometry of this Gauss point (k_geometry)
      const double* gp = a.geo + (size_t)e * GEO_PER_ELEM + g * GEO_PER_GP;
      const double w = gp[0];
      double dndx[6], dndy[6], dmdx[3], dmdy[3];
      for (int j = 0; j < 6; j++) {
        dndx[j] = gp[1 + j];
        dndy[j] = gp[7 + j];
        d.dndx[g][j] = dndx[j];
        d.dndy[g][j] = dndy[j];
        d.kdndx[g][j] = (KT)dndx[j];
        d.kdndy[g][j] = (KT)dndy[j];
      }
      for (int j = 0; j < 3; j++) {
        dmdx[j] = gp[13 + j];
        dmdy[j] = gp[16 + j];
        d.dmdx[g][j] = dmdx[j];
        d.dmdy[g][j] = dmdy[j];
        d.kdmdx[g][j] = (KT)dmdx[j];
        d.kdmdy[g][j] = (KT)dmdy[j];
      }
      double H = 0, dHdt = 0, dHdx = 0, dHdy = 0, dadx = 0, dady = 0, cf = 0;
      for (int j = 0; j < 3; j++) {
        double ndZ = d.nd[5][j];
        double ndH = d.nd[4][j] - ndZ;
        if (ndH <= 0.0) ndH = a.hmin;
        double mj = cS.m[g][j];
        H += mj * ndH;
        dHdx += dmdx[j] * ndH;
        dHdy += dmdy[j] * ndH;
        dadx += dmdx[j] * ndZ;
        dady += dmdy[j] * ndZ;
        dHdt += mj * d.nd[6][j];
        cf += mj * d.nd[7][j];
      }
      double U = 0, dUdt = 0, dUdx = 0, dUdy = 0, V = 0, dVdt = 0, dVdx = 0, dVdy = 0;
      for (int j = 0; j < 6; j++) {
        double nj = cS.n[g][j];
        double ndU = d.nd[0][j], ndV = d.nd[1][j];
        U += nj * ndU;
        dUdt += nj * d.nd[2][j];
        dUdx += dndx[j] * ndU;
        dUdy += dndy[j] * ndU;
        V += nj * ndV;
        dVdt += nj * d.nd[3][j];
        dVdx += dndx[j] * ndV;
        dVdy += dndy[j] * ndV;
      }
      const double vt = a.evt[e] + a.vk;
      const double gr = a.g;
      const double Ures = sqrt(U * U + V * V);
      // residual integrands (CoefsUVS2D.cpp:641-736)
      double ff, fx, fy;
      ff = H * dUdt + H * (U * dUdx + V * dUdy);
      fx = H * vt * (dUdx + dUdx);
      fy = H * vt * (dUdy + dVdx);
      ff += H * gr * dadx;
      fx -= H * H * gr / 2.0;
      ff += cf * Ures * U;
      d.res[g][0] = ff * w;
      d.res[g][1] = fx * w;
      d.res[g][2] = fy * w;
      ff = H * dVdt + H * (U * dVdx + V * dVdy);
      fx = H * vt * (dVdx + dUdy);
      fy = H * vt * (dVdy + dVdy);
      ff += H * gr * dady;
      fy -= H * H * gr / 2.0;
      ff += cf * Ures * V;
      d.res[g][3] = ff * w;
      d.res[g][4] = fx * w;
      d.res[g][5] = fy * w;
      d.res[g][6] = (dHdt + H * (dUdx + dVdy) + U * dHdx + V * dHdy) * w;
      // Jacobian block coefficients (CoefsUVS2D.cpp:749-1059)
      double iUres = (Ures > 1.0e-9) ? 1.0 / Ures : 0.0;
      if constexpr (sizeof(KT) == 4)
        block_coefs<float>(d.coef[g], (float)w, (float)H, (float)U, (float)V, (float)dUdx, (float)dUdy, (float)dVdx,
                           (float)dVdy, (float)dUdt, (float)dVdt, (float)dHdx, (float)dHdy, (float)dadx, (float)dady,
                           (float)cf, (float)Ures, (float)iUres, (float)vt, (float)gr, (float)a.rUV, (float)a.rH);
      else
        block_coefs<double>(d.coef[g], w, H, U, V, dUdx, dUdy, dVdx, dVdy, dUdt, dVdt, dHdx, dHdy, dadx, dady, cf,
                            Ures, iUres, vt, gr, a.rUV, a.rH);
    }
    __syncwarp();


    for (int j = 0; j < nel; j++) {
      const int p = a.reg[base + j];
      const int e = a.elems[p];
      const int* nd = a.enodes + 6 * e;
      GpData<KT>& d = s.el[j];
      bool have_area = false;

      // 3. trial vectors: 7 GP x 9 blocks x 6 columns (t, tx, ty), one block per
      // pass so that the block switch is warp-uniform
#pragma unroll 1
      for (int b = 0; b < 9; b++)
      for (int idx = lane; idx < 7 * 6; idx += 32) {
        const int g = idx / 6, k = idx % 6;
        const KT* c = d.coef[g];
        const KT nk = shape_n<KT>(g, k), xk = d.kdndx[g][k], yk = d.kdndy[g][k];
        KT t = 0, tx = 0, ty = 0;
        switch (b) {
          case 0:  // U row, U col
            t = c[C_UU0] * nk + c[C_UUX] * xk + c[C_UUY] * yk;
            tx = c[C_UUXX] * xk;
            ty = c[C_UUYY] * yk;
            break;
          case 1:  // U row, V col
            t = c[C_UV0] * nk;
            ty = c[C_UVYX] * xk;
            break;
          case 2:  // U row, H col (corners)
            if (k < 3) {
              KT mk = shape_m<KT>(g, k);
              t = (c[C_UH0] + c[C_UF] * d.dcf[k]) * mk;
              tx = c[C_UHX] * mk;
              ty = c[C_UHY] * mk;
            }
            break;
          case 3:  // V row, U col
            t = c[C_VU0] * nk;
            tx = c[C_VUXY] * yk;
            break;
          case 4:  // V row, V col
            t = c[C_VV0] * nk + c[C_VVX] * xk + c[C_VVY] * yk;
            tx = c[C_VVXX] * xk;
            ty = c[C_VVYY] * yk;
            break;
          case 5:  // V row, H col
            if (k < 3) {
              KT mk = shape_m<KT>(g, k);
              t = (c[C_VH0] + c[C_VF] * d.dcf[k]) * mk;
              tx = c[C_VHX] * mk;
              ty = c[C_VHY] * mk;
            }
            break;
          case 6:  // S row, U col
            t = c[C_SU0] * nk + c[C_SUX] * xk;
            break;
          case 7:  // S row, V col
            t = c[C_SV0] * nk + c[C_SVY] * yk;
            break;
          case 8:  // S row, H col
            if (k < 3) {
              t = c[C_SH0] * shape_m<KT>(g, k) + c[C_SHX] * d.kdmdx[g][k] + c[C_SHY] * d.kdmdy[g][k];
            }
            break;
        }
        s.T[g][b][0][k] = t;
        s.T[g][b][1][k] = tx;
        s.T[g][b][2][k] = ty;
      }
      __syncwarp();

      // 4. element matrix and residual
      for (int idx = lane; idx < RG_EQ * RG_EQ; idx += 32) {
        const int r = idx / RG_EQ, cc = idx % RG_EQ;
        const int rv = (r < 6) ? 0 : (r < 12 ? 1 : 2), j = r - 6 * rv;
        const int cv = (cc < 6) ? 0 : (cc < 12 ? 1 : 2), k = cc - 6 * cv;
        const int b = rv * 3 + cv;
        KT acc = 0;
        if (k < 6 && !(cv == 2 && k >= 3)) {
          for (int g = 0; g < 7; g++) {
            if (rv < 2) {
              acc += shape_n<KT>(g, j) * s.T[g][b][0][k] + d.kdndx[g][j] * s.T[g][b][1][k] +
                     d.kdndy[g][j] * s.T[g][b][2][k];
            } else {
              acc += shape_m<KT>(g, j) * s.T[g][b][0][k];
            }
          }
        }
        s.K[r][cc] = acc;
      }
      if (lane < RG_EQ) {
        const int r = lane;
        double acc = 0.0;
        if (r < 12) {
          const int o = (r < 6) ? 0 : 3, j = (r < 6) ? r : r - 6;
          for (int g = 0; g < 7; g++)
            acc -= cS.n[g][j] * d.res[g][o] + d.dndx[g][j] * d.res[g][o + 1] + d.dndy[g][j] * d.res[g][o + 2];
        } else {
          const int j = r - 12;
          for (int g = 0; g < 7; g++) acc -= cS.m[g][j] * d.res[g][6];
        }
        s.f[r] = acc;
      }
      __syncwarp();

      // 5. boundary rotation (Rotate.cpp:42-107), node by node
      for (int i = 0; i < 6; i++) {
        const int n = nd[i];
        if (!(a.nflag[n] & RG_N_ROTAT)) continue;
        const double r00 = a.rot[4 * n], r01 = a.rot[4 * n + 1], r10 = a.rot[4 * n + 2], r11 = a.rot[4 * n + 3];
        const double det = r00 * r11 - r01 * r10;
        if (fabs(det) < 1.0e-12) continue;
        const int j = 6 + i;
        if (lane < RG_EQ) {
          KT ki = s.K[lane][i], kj = s.K[lane][j];
          s.K[lane][i] = ki * (KT)r00 + kj * (KT)r10;
          s.K[lane][j] = ki * (KT)r01 + kj * (KT)r11;
        }
        __syncwarp();
        if (lane < RG_EQ) {
          KT ki = s.K[i][lane], kj = s.K[j][lane];
          s.K[i][lane] = (KT)r00 * ki + (KT)r10 * kj;
          s.K[j][lane] = (KT)r01 * ki + (KT)r11 * kj;
        }
        if (lane == 0) {
          double fi = s.f[i], fj = s.f[j];
          s.f[i] = r00 * fi + r10 * fj;
          s.f[j] = r01 * fi + r11 * fj;
        }
        __syncwarp();
      }

      // 6. inlet rows (CoefsUVS2D.cpp:1078-1181)
      for (int i = 0; i < 6; i++) {
        const int k = nd[i];
        if (!(a.bckind[k] & RG_B_INLET)) continue;
        double Un = a.U[k] * a.niox[k] + a.V[k] * a.nioy[k];
        double H, specQ = a.bcU[k];
        int l = -1, r = -1;
        if (i < 3) {
          H = a.S[k] - a.z[k];
        } else {
          l = i - 3;
          r = (i - 2) % 3;
          double Hl = d.nd[4][l] - d.nd[5][l], Hr = d.nd[4][r] - d.nd[5][r];
          H = (Hl + Hr) / 2.0;
        }
        if (H <= 0.0) {
          H = a.hmin;
          specQ = 0.0;
        }
        if (lane < RG_EQ) s.K[i][lane] = 0;
        __syncwarp();
        if (lane == 0) {
          if (!have_area) {  // element area in FP64 regardless of KT (sum of GP weights)
            double x[6], y[6];
            x[0] = 0.0;
            y[0] = 0.0;
            for (int i = 1; i < 6; i++) {
              x[i] = d.nd[8][i] - d.nd[8][0];
              y[i] = d.nd[9][i] - d.nd[9][0];
            }
            double area = 0.0;
            for (int g = 0; g < 7; g++) {
              double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
              for (int k = 0; k < 6; k++) {
                j00 += cS.dnx[g][k] * x[k];
                j01 += cS.dnx[g][k] * y[k];
                j10 += cS.dny[g][k] * x[k];
                j11 += cS.dny[g][k] * y[k];
              }
              area += (j00 * j11 - j01 * j10) * cS.w[g];
            }
            s.area = area;
            have_area = true;
          }
          s.f[i] = s.area * (specQ - Un * H);
          s.K[i][i] = (KT)(s.area * H);
          if (i < 3) {
            s.K[i][12 + i] = (KT)(s.area * Un);
          } else {
            s.K[i][12 + l] = (KT)(s.area * Un / 2.0);
            s.K[i][12 + r] = (KT)(s.area * Un / 2.0);
          }
        }
        __syncwarp();
      }

      // 7. store by assembly position
      KT* ek = EK + (size_t)p * (RG_EQ * RG_EQ);
      for (int idx = lane; idx < RG_EQ * RG_EQ; idx += 32) ek[idx] = s.K[idx / RG_EQ][idx % RG_EQ];
      if (lane < RG_EQ) EF[(size_t)p * RG_EQ + lane] = s.f[lane];
      __syncwarp();
    }
  }
}

// Phase 2: each CRS value and each residual row is the sum of its element
// contributions in assembly order -- the values and the rounding of the
// reference's element-by-element scatter (Assemble.cpp:256-343), with no
// atomics and every entry written once.
template <class KT, class MT>
__global__ void k_asm_gather(long long nnz, const long long* __restrict__ gptr, const int* __restrict__ gsrc,
                             const KT* __restrict__ EK, MT* __restrict__ A, int neq,
                             const long long* __restrict__ rptr, const int* __restrict__ rsrc,
                             const double* __restrict__ EF, double* __restrict__ B) {
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < nnz + neq;
       t += (long long)gridDim.x * blockDim.x) {
    if (t < nnz) {
      MT acc = (MT)0;
      for (long long k = gptr[t]; k < gptr[t + 1]; k++) acc += (MT)EK[gsrc[k]];
      A[t] = acc;
    } else {
      const int r = (int)(t - nnz);
      double acc = 0.0;
      for (long long k = rptr[r]; k < rptr[r + 1]; k++) acc += EF[rsrc[k]];
      B[r] = acc;
    }
  }
}

__global__ void k_pow_third(double h, double* out) { *out = pow(h, 0.333333); }

// nodal Manning friction, gathered per node over its region triangles in
// element order (DoFriction.cpp:87-206)
__global__ void k_friction(int np, const int* __restrict__ nptr, const int* __restrict__ nel,
                           const double* __restrict__ elem_n, const double* __restrict__ elem_af,
                           const double* __restrict__ S, const double* __restrict__ z, double hmin, double g,
                           const double* __restrict__ phmin, double* __restrict__ cf) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= np) return;
  int b = nptr[k], e = nptr[k + 1];
  if (b == e) {
    cf[k] = 0.0;
    return;
  }
  double h = S[k] - z[k];
  // depth clipped to hmin (every dry node): the same pow, evaluated once per context
  const double ph = (h <= hmin) ? *phmin : pow(h, 0.333333);
  double acc = 0.0;
  for (int q = b; q < e; q++) {
    int el = nel[q];
    double rc = elem_n[el];
    acc += elem_af[el] * (g * (rc * rc) / ph);
  }
  cf[k] = acc / (double)(e - b);
}

bool g_tables_ready[64] = {false};

}  // namespace

cudaError_t launch_assemble(rg_ctx* c) {
  if (c->device >= 0 && c->device < 64 && !g_tables_ready[c->device]) {
    ShapeTables t = make_tables();
    cudaError_t e = cudaMemcpyToSymbol(cS, &t, sizeof(t));
    if (e != cudaSuccess) return e;
    ShapeTablesF tf;
    for (int g = 0; g < 7; g++) {
      for (int k = 0; k < 6; k++) tf.n[g][k] = (float)t.n[g][k];
      for (int k = 0; k < 3; k++) tf.m[g][k] = (float)t.m[g][k];
    }
    e = cudaMemcpyToSymbol(cSf, &tf, sizeof(tf));
    if (e != cudaSuccess) return e;
    g_tables_ready[c->device] = true;
  }
  AsmArgs a;
  a.x = c->x.p; a.y = c->y.p; a.z = c->z.p; a.U = c->U.p; a.V = c->V.p; a.S = c->S.p;
  a.dUdt = c->dUdt.p; a.dVdt = c->dVdt.p; a.dSdt = c->dSdt.p; a.cf = c->cf.p; a.cfw = c->cfw.p;
  a.nflag = c->nflag.p; a.bckind = c->bckind.p; a.rot = c->rot.p; a.niox = c->niox.p; a.nioy = c->nioy.p;
  a.bcU = c->bcU.p; a.bcS = c->bcS.p; a.enodes = c->enodes.p; a.eflag = c->eflag.p;
  a.evt = c->evt.p; a.g = c->g; a.hmin = c->hmin; a.vk = c->vk; a.rUV = c->rUV; a.rH = c->rH;
  a.jac_friction = c->jac_friction;
  a.elems = c->color_elem.p;
  a.reg = c->asm_reg.p;
  a.count = c->n_asm_reg;
  a.bnd = c->asm_bnd.p;
  a.bcount = c->n_asm_bnd;
  if (!c->geo_valid) {
    cudaError_t e = c->geo.alloc((size_t)std::max(c->ne, 1) * GEO_PER_ELEM);
    if (e != cudaSuccess) return e;
    if (a.count > 0) {
      const int gblocks = std::min((a.count * 7 + 127) / 128, c->num_sms * 8);
      if (c->prec == RG_PREC_MIXED)
        k_geometry<float><<<gblocks, 128, 0, rg_counted(c)>>>(a, c->geo.p);
      else
        k_geometry<double><<<gblocks, 128, 0, rg_counted(c)>>>(a, c->geo.p);
    }
    c->geo_valid = true;
  }
  a.geo = c->geo.p;
  constexpr int EPW = 4;
  const int items = (a.count + EPW - 1) / EPW + a.bcount;
  const long long ntot = (long long)c->nnz + c->neq;
  const int gb = (int)std::min<long long>((ntot + 255) / 256, (long long)c->num_sms * 16);
  // shared memory per warp: ~26 KB with FP64 element matrices, ~17 KB with FP32
  if (c->prec == RG_PREC_MIXED) {
    if (items > 0) {
      const int blocks = std::min((items + 1) / 2, c->num_sms * 6);
      k_element<float, 2, EPW><<<blocks, 64, 0, rg_counted(c)>>>(a, c->EK32.p, c->EF.p);
    }
    k_asm_gather<float, float><<<gb, 256, 0, rg_counted(c)>>>(c->nnz, c->gat_ptr.p, c->gat_src.p, c->EK32.p,
                                                               c->A32.p, c->neq, c->grow_ptr.p, c->grow_src.p,
                                                               c->EF.p, c->B.p);
  } else {
    if (items > 0) {
      const int blocks = std::min(items, c->num_sms * 8);
      k_element<double, 1, EPW><<<blocks, 32, 0, rg_counted(c)>>>(a, c->EK64.p, c->EF.p);
    }
    if (c->prec == RG_PREC_FP64)
      k_asm_gather<double, double><<<gb, 256, 0, rg_counted(c)>>>(c->nnz, c->gat_ptr.p, c->gat_src.p, c->EK64.p,
                                                                   c->A64.p, c->neq, c->grow_ptr.p, c->grow_src.p,
                                                                   c->EF.p, c->B.p);
    else
      k_asm_gather<double, float><<<gb, 256, 0, rg_counted(c)>>>(c->nnz, c->gat_ptr.p, c->gat_src.p, c->EK64.p,
                                                                  c->A32.p, c->neq, c->grow_ptr.p, c->grow_src.p,
                                                                  c->EF.p, c->B.p);
  }
  return cudaGetLastError();
}

cudaError_t launch_friction(rg_ctx* c) {
  int np = c->np;
  if (c->fr_phmin_h != c->hmin) {
    cudaError_t e = c->fr_phmin.alloc(1);
    if (e != cudaSuccess) return e;
    k_pow_third<<<1, 1, 0, rg_counted(c)>>>(c->hmin, c->fr_phmin.p);
    c->fr_phmin_h = c->hmin;
  }
  k_friction<<<(np + 255) / 256, 256, 0, rg_counted(c)>>>(np, c->fr_ptr.p, c->fr_el.p, c->elem_n.p, c->elem_af.p,
                                                   c->S.p, c->z.p, c->hmin, c->g, c->fr_phmin.p, c->cf.p);
  return cudaGetLastError();
}
