/*
 * CPU restatement of the reference's shallow-water Newton step (parity oracle).
 * TEST INFRASTRUCTURE ONLY -- see rg_oracle.h.  Never linked into the library.
 */
#include "rg_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

/* flags (Node.h, Elem.h, Bcon.h) */
#define N_ROTAT     32
#define E_INLET      1
#define E_OUTLET     2
#define E_OPENBND    4
#define E_BOUND     16
#define E_DRY      128
#define B_INLET      1
#define B_OUTLET     2
#define B_OPENBND    4
#define B_LOGLAW   256
#define B_SOURCE  2048

#define MAXEQ 24          /* maxEleq = 3 dof x kMaxNodes2D */

/* ------------------------------------------------------------------------ */
/* shape functions at the Gauss points of degree 5 (Shape.cpp:89-205,
 * 308-322; Triangle.cpp:43-327; Line.cpp:43-152)                            */

static double tri_w[7], tri_m[7][3], tri_dmx[7][3], tri_dmy[7][3];
static double tri_n[7][6], tri_dnx[7][6], tri_dny[7][6];
static double lin_w[3], lin_m[3][2], lin_n[3][3], lin_dn[3][3];
static int shapes_ready = 0;

static void init_shapes(void)
{
  if( shapes_ready ) return;
  static const double loc[7][2] = {
    { 1.0/3.0, 1.0/3.0 },
    { 0.0597158717897698, 0.470142064105115 },
    { 0.470142064105115,  0.0597158717897698 },
    { 0.470142064105115,  0.470142064105115 },
    { 0.797426985353087,  0.101286507323456 },
    { 0.101286507323456,  0.797426985353087 },
    { 0.101286507323456,  0.101286507323456 } };
  static const double w[7] = { 0.1125, 0.0661970763942531, 0.0661970763942531, 0.0661970763942531,
                               0.0629695902724136, 0.0629695902724136, 0.0629695902724136 };
  for( int g=0; g<7; g++ )
  {
    double xi = loc[g][0], et = loc[g][1];
    double L[3] = { 1.0 - xi - et, xi, et };
    double dLx[3] = { -1.0, 1.0, 0.0 }, dLy[3] = { -1.0, 0.0, 1.0 };
    tri_w[g] = w[g];
    for( int i=0; i<3; i++ )
    {
      tri_m[g][i] = L[i];  tri_dmx[g][i] = dLx[i];  tri_dmy[g][i] = dLy[i];
      tri_n[g][i]   = (2.0*L[i] - 1.0) * L[i];
      tri_dnx[g][i] = (4.0*L[i] - 1.0) * dLx[i];
      tri_dny[g][i] = (4.0*L[i] - 1.0) * dLy[i];
    }
    for( int k=3; k<6; k++ )
    {
      int i = k % 3, j = (k + 1) % 3;
      tri_n[g][k]   = 4.0 * L[i] * L[j];
      tri_dnx[g][k] = 4.0 * (dLx[i] * L[j] + L[i] * dLx[j]);
      tri_dny[g][k] = 4.0 * (dLy[i] * L[j] + L[i] * dLy[j]);
    }
  }
  for( int g=0; g<3; g++ )
  {
    double x = (g == 0) ? -sqrt(0.6) : (g == 1 ? 0.0 : sqrt(0.6));
    lin_w[g] = (g == 1) ? 8.0/9.0 : 5.0/9.0;
    lin_m[g][0] = (1.0 - x) / 2.0;  lin_m[g][1] = (1.0 + x) / 2.0;
    lin_n[g][0] = x * (x - 1.0) / 2.0;  lin_n[g][1] = x * (x + 1.0) / 2.0;  lin_n[g][2] = 1.0 - x*x;
    lin_dn[g][0] = x - 0.5;  lin_dn[g][1] = x + 0.5;  lin_dn[g][2] = -2.0 * x;
  }
  shapes_ready = 1;
}

/* the derivative of the P2 triangle shape functions is restated from the
 * product rule; Triangle.cpp:330-400 evaluates the same polynomials */

/* ------------------------------------------------------------------------ */
/* EQS::Rotate2D (Rotate.cpp:42-107)                                          */

static void rotate2d(const orc_model* m, int nnd, const int* nd, double* K, double* f)
{
  int eqid = nnd;
  for( int i=0; i<nnd; i++ )
  {
    int n = nd[i];
    if( !(m->nflag[n] & N_ROTAT) ) continue;
    const double* r = m->rot + 4*n;
    double r00 = r[0], r01 = r[1], r10 = r[2], r11 = r[3];
    double det = r00*r11 - r01*r10;
    if( fabs(det) < 1.0e-12 ) continue;
    int j = eqid + i;
    if( K )
    {
      for( int k=0; k<MAXEQ; k++ )
      {
        double tmp     = K[k*MAXEQ+i] * r00  +  K[k*MAXEQ+j] * r10;
        K[k*MAXEQ+j]   = K[k*MAXEQ+i] * r01  +  K[k*MAXEQ+j] * r11;
        K[k*MAXEQ+i]   = tmp;
      }
      for( int k=0; k<MAXEQ; k++ )
      {
        double tmp     = r00 * K[i*MAXEQ+k]  +  r10 * K[j*MAXEQ+k];
        K[j*MAXEQ+k]   = r01 * K[i*MAXEQ+k]  +  r11 * K[j*MAXEQ+k];
        K[i*MAXEQ+k]   = tmp;
      }
    }
    if( f )
    {
      double tmp = r00 * f[i]  +  r10 * f[j];
      f[j]       = r01 * f[i]  +  r11 * f[j];
      f[i]       = tmp;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* EQS_UVS2D::Bound (CoefsUVS2D.cpp:71-360): 3-node boundary line            */

static void coefs_bound(const orc_model* m, int e, double* K, double* f)
{
  const int* nd = m->enodes + 6*e;
  const int nnd = 3, eqidV = 3, eqidS = 6;
  double gravity = m->g;
  memset( f, 0, MAXEQ*sizeof(double) );
  memset( K, 0, MAXEQ*MAXEQ*sizeof(double) );
  int fl = m->eflag[e];
  int solid = !(  !(m->bckind[nd[2]] & B_LOGLAW) || (fl & E_INLET) || (fl & E_OUTLET) || (fl & E_OPENBND) );
  int outlet = (m->bckind[nd[2]] & B_OUTLET) != 0;
  for( int g=0; g<3; g++ )
  {
    const double* mm = lin_m[g];
    const double* n  = lin_n[g];
    const double* dn = lin_dn[g];
    double H0, H1;
    if( outlet ) { H0 = m->bcS[nd[0]] - m->z[nd[0]];  H1 = m->bcS[nd[1]] - m->z[nd[1]]; }
    else         { H0 = m->S[nd[0]]   - m->z[nd[0]];  H1 = m->S[nd[1]]   - m->z[nd[1]]; }
    if( H0 <= 0.0 ) H0 = m->hmin;
    if( H1 <= 0.0 ) H1 = m->hmin;
    double H = mm[0]*H0 + mm[1]*H1;
    double nx =  dn[0]*m->y[nd[0]] + dn[1]*m->y[nd[1]] + dn[2]*m->y[nd[2]];
    double ny = -dn[0]*m->x[nd[0]] - dn[1]*m->x[nd[1]] - dn[2]*m->x[nd[2]];
    double len = sqrt( nx*nx + ny*ny );
    double weight = lin_w[g];
    double U = 0.0, V = 0.0, Ures = 0.0, cf = 0.0;
    if( solid )
    {
      U = n[0]*m->U[nd[0]] + n[1]*m->U[nd[1]] + n[2]*m->U[nd[2]];
      V = n[0]*m->V[nd[0]] + n[1]*m->V[nd[1]] + n[2]*m->V[nd[2]];
      Ures = sqrt( U*U + V*V );
      cf = mm[0]*m->cfw[nd[0]] + mm[1]*m->cfw[nd[1]];
    }
    double fU = weight * H * ( gravity*H/2.0 * nx );
    double fV = weight * H * ( gravity*H/2.0 * ny );
    if( solid )
    {
      fU += weight * len * H * cf * U * Ures;
      fV += weight * len * H * cf * V * Ures;
    }
    for( int i=0; i<3; i++ ) { f[i] -= n[i] * fU;  f[eqidV+i] -= n[i] * fV; }

    double dfUdU = 0, dfUdV = 0, dfUdH = 0, dfVdU = 0, dfVdV = 0, dfVdH = 0;
    if( !outlet )
    {
      dfUdH += weight * ( gravity*H * nx );
      dfVdH += weight * ( gravity*H * ny );
    }
    if( solid )
    {
      dfUdH += weight * len * cf * U * Ures;
      dfVdH += weight * len * cf * V * Ures;
      double iUres = ( Ures > 1.0e-8 ) ? 1.0 / Ures : 0.0;
      dfUdU += weight * len * cf * H * (U * U * iUres  +  Ures);
      dfUdV += weight * len * cf * H * (U * V * iUres);
      dfVdU += weight * len * cf * H * (U * V * iUres);
      dfVdV += weight * len * cf * H * (V * V * iUres  +  Ures);
    }
    for( int i=0; i<3; i++ )
    {
      for( int k=0; k<3; k++ )
      {
        K[i*MAXEQ + k]                 += n[i] * dfUdU * n[k];
        K[i*MAXEQ + eqidV + k]         += n[i] * dfUdV * n[k];
        K[(eqidV+i)*MAXEQ + k]         += n[i] * dfVdU * n[k];
        K[(eqidV+i)*MAXEQ + eqidV + k] += n[i] * dfVdV * n[k];
      }
      for( int k=0; k<2; k++ )
      {
        K[i*MAXEQ + eqidS + k]         += n[i] * dfUdH * mm[k];
        K[(eqidV+i)*MAXEQ + eqidS + k] += n[i] * dfVdH * mm[k];
      }
    }
  }
  rotate2d( m, nnd, nd, K, f );
  for( int i=0; i<nnd; i++ )
  {
    if( m->bckind[nd[i]] & B_INLET )
    {
      for( int j=0; j<MAXEQ; j++ ) K[i*MAXEQ+j] = 0.0;
      f[i] = 0.0;
    }
  }
}

/* ------------------------------------------------------------------------ */
/* EQS_UVS2D::Region (CoefsUVS2D.cpp:365-1182): six-node triangle, 7 GPs     */

static void coefs_region(const orc_model* m, int e, double* K, double* f)
{
  const int* nd = m->enodes + 6*e;
  const int nnd = 6, ncn = 3, eqidV = 6, eqidS = 12;
  memset( f, 0, MAXEQ*sizeof(double) );
  memset( K, 0, MAXEQ*MAXEQ*sizeof(double) );
  double gravity = m->g;
  double rUV = m->relaxThdt_UV, rH = m->relaxThdt_H;
  double area = 0.0;
  double x[6], y[6];
  x[0] = m->x[nd[0]];  y[0] = m->y[nd[0]];
  for( int i=1; i<nnd; i++ ) { x[i] = m->x[nd[i]] - x[0];  y[i] = m->y[nd[i]] - y[0]; }
  x[0] = y[0] = 0.0;
  double vt0 = m->evt[e] + m->vk;       /* kVtConstant: type->vt, plus vk */

  for( int g=0; g<7; g++ )
  {
    const double *dfdx = tri_dnx[g], *dfdy = tri_dny[g];
    double j00 = 0, j01 = 0, j10 = 0, j11 = 0;
    for( int k=0; k<nnd; k++ )
    {
      j00 += dfdx[k] * x[k];  j01 += dfdx[k] * y[k];
      j10 += dfdy[k] * x[k];  j11 += dfdy[k] * y[k];
    }
    double detj = j00*j11 - j01*j10;
    double t00 = j11/detj, t01 = -j01/detj, t10 = -j10/detj, t11 = j00/detj;
    double weight = detj * tri_w[g];
    area += weight;
    double dndx[6], dndy[6];
    const double* n = tri_n[g];
    for( int j=0; j<nnd; j++ )
    {
      dndx[j] = t00*dfdx[j] + t01*dfdy[j];
      dndy[j] = t10*dfdx[j] + t11*dfdy[j];
    }
    double dmdx[3], dmdy[3];
    const double* mm = tri_m[g];
    for( int j=0; j<ncn; j++ )
    {
      dmdx[j] = t00*tri_dmx[g][j] + t01*tri_dmy[g][j];
      dmdy[j] = t10*tri_dmx[g][j] + t11*tri_dmy[g][j];
    }
    double H = 0, dHdt = 0, dHdx = 0, dHdy = 0, dadx = 0, dady = 0, cf = 0, SS = 0;
    for( int j=0; j<ncn; j++ )
    {
      int k = nd[j];
      double ndZ = m->z[k];
      double ndH = m->S[k] - ndZ;
      if( ndH <= 0.0 ) ndH = m->hmin;
      double ndSS = 0.0;   /* kSource is not used by the supported decks */
      H    +=    mm[j] * ndH;
      dHdx += dmdx[j] * ndH;
      dHdy += dmdy[j] * ndH;
      dadx += dmdx[j] * ndZ;
      dady += dmdy[j] * ndZ;
      dHdt +=    mm[j] * m->dSdt[k];
      cf   +=    mm[j] * m->cf[k];
      SS   +=    mm[j] * ndSS;
    }
    double U = 0, dUdt = 0, dUdx = 0, dUdy = 0, V = 0, dVdt = 0, dVdx = 0, dVdy = 0;
    double uu = 0, uv = 0, vv = 0;
    for( int j=0; j<nnd; j++ )
    {
      int k = nd[j];
      double ndU = m->U[k], ndV = m->V[k];
      U    +=    n[j] * ndU;  dUdt += n[j] * m->dUdt[k];
      dUdx += dndx[j] * ndU;  dUdy += dndy[j] * ndU;
      V    +=    n[j] * ndV;  dVdt += n[j] * m->dVdt[k];
      dVdx += dndx[j] * ndV;  dVdy += dndy[j] * ndV;
      uu += n[j] * m->uu[k];  uv += n[j] * m->uv[k];  vv += n[j] * m->vv[k];
    }
    const double Dxx = 0.0, Dxy = 0.0, Dyy = 0.0;    /* actualDisp == 0 */
    double vt = vt0;
    double Ures = sqrt( U*U + V*V );

    /* residual */
    {
      double ff, fx, fy;
      ff  = H * dUdt;
      ff += H * (U * dUdx + V * dUdy);
      fx  = H * vt * (dUdx + dUdx);
      fy  = H * vt * (dUdy + dVdx);
      fx -= H * uu;
      fy -= H * uv;
      ff += H * gravity * dadx;
      fx -= H * H * gravity / 2.0;
      ff += cf * Ures * U;
      fx += H * ( U*U*Dxx - 2.0*U*V*Dxy + V*V*Dyy );
      fy += H * ( U*V*(Dxx-Dyy) + (U*U-V*V)*Dxy );
      ff *= weight;  fx *= weight;  fy *= weight;
      for( int j=0; j<nnd; j++ ) f[j] -= n[j]*ff + dndx[j]*fx + dndy[j]*fy;

      ff  = H * dVdt;
      ff += H * (U * dVdx + V * dVdy);
      fx  = H * vt * (dVdx + dUdy);
      fy  = H * vt * (dVdy + dVdy);
      fx -= H * uv;
      fy -= H * vv;
      ff += H * gravity * dady;
      fy -= H * H * gravity / 2.0;
      ff += cf * Ures * V;
      fx += H * ( U*V*(Dxx-Dyy) + (U*U-V*V)*Dxy );
      fy += H * ( V*V*Dxx + 2.0*U*V*Dxy + U*U*Dyy );
      ff *= weight;  fx *= weight;  fy *= weight;
      for( int j=0; j<nnd; j++ ) f[eqidV+j] -= n[j]*ff + dndx[j]*fx + dndy[j]*fy;

      ff  = dHdt + H * (dUdx + dVdy) + U * dHdx + V * dHdy;
      ff += SS;
      ff *= weight;
      for( int j=0; j<ncn; j++ ) f[eqidS+j] -= mm[j] * ff;
    }

    /* Jacobian */
    {
      double t[6], tx[6], ty[6];
      double df__, df_x, df_y, dfx_, dfy_, dfxx, dfyy, dfxy, dfyx;
      double iUres = ( Ures > 1.0e-9 ) ? 1.0 / Ures : 0.0;

      /* U-derivative of x-momentum */
      df__  = weight * H * rUV;
      df__ += weight * H * dUdx;
      df_x  = weight * H * U;
      df_y  = weight * H * V;
      dfx_  = 0.0;  dfy_ = 0.0;
      dfxx  = weight * H * vt * 2.0;
      dfyy  = weight * H * vt;
      df__ += weight * cf * (iUres * U*U + Ures);
      dfx_ += weight * H * ( 2.0*U*Dxx - 2.0*V*Dxy );
      dfy_ += weight * H * ( V*(Dxx-Dyy) + 2.0*U*Dxy );
      for( int j=0; j<nnd; j++ )
      {
        t[j]  = df__*n[j] + df_x*dndx[j] + df_y*dndy[j];
        tx[j] = dfx_*n[j] + dfxx*dndx[j];
        ty[j] = dfy_*n[j] + dfyy*dndy[j];
      }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<nnd; k++ )
          K[j*MAXEQ + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* V-derivative of x-momentum */
      df__  = weight * H * dUdy;
      dfx_  = 0.0;  dfy_ = 0.0;
      dfyx  = weight * H * vt;
      df__ += weight * cf * iUres * U * V;
      dfx_ += weight * H * ( 2.0*V*Dyy - 2.0*V*Dxy );
      dfy_ += weight * H * ( V*(Dxx-Dyy) - 2.0*V*Dxy );
      for( int j=0; j<nnd; j++ )
      {
        t[j]  = df__*n[j];
        tx[j] = dfx_*n[j];
        ty[j] = dfy_*n[j] + dfyx*dndx[j];
      }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<nnd; k++ )
          K[j*MAXEQ + eqidV + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* H-derivative of x-momentum */
      df__  = weight * dUdt;
      df__ += weight * (U * dUdx + V * dUdy);
      dfx_  = 0.0;  dfy_ = 0.0;
      dfx_ += weight * vt * (dUdx + dUdx);
      dfy_ += weight * vt * (dUdy + dVdx);
      dfx_ -= weight * uu;
      dfy_ -= weight * uv;
      df__ += weight * gravity * dadx;
      dfx_ -= weight * gravity * H;
      dfx_ += weight * ( U*U*Dxx - 2.0*U*V*Dxy + V*V*Dyy );
      dfy_ += weight * ( U*V*(Dxx-Dyy) + (U*U-V*V)*Dxy );
      for( int j=0; j<ncn; j++ ) { t[j] = df__*mm[j];  tx[j] = dfx_*mm[j];  ty[j] = dfy_*mm[j]; }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<ncn; k++ )
          K[j*MAXEQ + eqidS + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* U-derivative of y-momentum */
      df__  = weight * H * dVdx;
      dfx_  = 0.0;  dfy_ = 0.0;
      dfxy  = weight * H * vt;
      df__ += weight * cf * iUres * U * V;
      dfx_ += weight * H * ( V*(Dxx-Dyy) + 2.0*U*Dxy );
      dfy_ += weight * H * ( 2.0*V*Dxy + 2.0*U*Dyy );
      for( int j=0; j<nnd; j++ )
      {
        t[j]  = df__*n[j];
        tx[j] = dfx_*n[j] + dfxy*dndy[j];
        ty[j] = dfy_*n[j];
      }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<nnd; k++ )
          K[(j+eqidV)*MAXEQ + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* V-derivative of y-momentum */
      df__  = weight * H * rUV;
      df__ += weight * H * dVdy;
      df_x  = weight * H * U;
      df_y  = weight * H * V;
      dfx_  = 0.0;  dfy_ = 0.0;
      dfxx  = weight * H * vt;
      dfyy  = weight * H * vt * 2.0;
      df__ += weight * cf * (iUres * V*V + Ures);
      dfx_ += weight * H * ( U*(Dxx-Dyy) - 2.0*V*Dxy );
      dfy_ += weight * H * ( 2.0*V*Dxx + 2.0*U*Dxy );
      for( int j=0; j<nnd; j++ )
      {
        t[j]  = df__*n[j] + df_x*dndx[j] + df_y*dndy[j];
        tx[j] = dfx_*n[j] + dfxx*dndx[j];
        ty[j] = dfy_*n[j] + dfyy*dndy[j];
      }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<nnd; k++ )
          K[(j+eqidV)*MAXEQ + eqidV + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* H-derivative of y-momentum */
      df__  = weight * dVdt;
      df__ += weight * (U * dVdx + V * dVdy);
      dfx_  = 0.0;  dfy_ = 0.0;
      dfx_ += weight * vt * (dVdx + dUdy);
      dfy_ += weight * vt * (dVdy + dVdy);
      dfx_ -= weight * uv;
      dfy_ -= weight * vv;
      df__ += weight * gravity * dady;
      dfy_ -= weight * gravity * H;
      dfx_ += weight * ( U*V*(Dxx-Dyy) + (U*U-V*V)*Dxy );
      dfy_ += weight * ( V*V*Dxx + 2.0*U*V*Dxy + U*U*Dyy );
      for( int j=0; j<ncn; j++ ) { t[j] = df__*mm[j];  tx[j] = dfx_*mm[j];  ty[j] = dfy_*mm[j]; }
      for( int j=0; j<nnd; j++ )
        for( int k=0; k<ncn; k++ )
          K[(j+eqidV)*MAXEQ + eqidS + k] += n[j]*t[k] + dndx[j]*tx[k] + dndy[j]*ty[k];

      /* U-derivative of continuity */
      df__ = weight * dHdx;
      df_x = weight * H;
      for( int j=0; j<nnd; j++ ) t[j] = df__*n[j] + df_x*dndx[j];
      for( int j=0; j<ncn; j++ )
        for( int k=0; k<nnd; k++ )
          K[(j+eqidS)*MAXEQ + k] += mm[j]*t[k];

      /* V-derivative of continuity */
      df__ = weight * dHdy;
      df_y = weight * H;
      for( int j=0; j<nnd; j++ ) t[j] = df__*n[j] + df_y*dndy[j];
      for( int j=0; j<ncn; j++ )
        for( int k=0; k<nnd; k++ )
          K[(j+eqidS)*MAXEQ + eqidV + k] += mm[j]*t[k];

      /* H-derivative of continuity */
      df__  = weight * rH;
      df__ += weight * (dUdx + dVdy);
      df_x  = weight * U;
      df_y  = weight * V;
      for( int j=0; j<ncn; j++ ) t[j] = df__*mm[j] + df_x*dmdx[j] + df_y*dmdy[j];
      for( int j=0; j<ncn; j++ )
        for( int k=0; k<ncn; k++ )
          K[(j+eqidS)*MAXEQ + eqidS + k] += mm[j]*t[k];
    }
  }

  rotate2d( m, nnd, nd, K, f );

  /* inlet rows: corner nodes (CoefsUVS2D.cpp:1078-1119) */
  for( int i=0; i<ncn; i++ )
  {
    int k = nd[i];
    if( !(m->bckind[k] & B_INLET) ) continue;
    for( int j=0; j<MAXEQ; j++ ) K[i*MAXEQ+j] = 0.0;
    double Un = m->U[k]*m->niox[k] + m->V[k]*m->nioy[k];
    double H = m->S[k] - m->z[k];
    double specQ = m->bcU[k];
    if( H <= 0.0 ) { H = m->hmin;  specQ = 0.0; }
    f[i] = area * (specQ - Un*H);
    K[i*MAXEQ + i]         = area * H;
    K[i*MAXEQ + i + eqidS] = area * Un;
  }
  /* inlet rows: mid-side nodes (CoefsUVS2D.cpp:1121-1181) */
  for( int i=ncn; i<nnd; i++ )
  {
    int k = nd[i];
    if( !(m->bckind[k] & B_INLET) ) continue;
    int l = i - 3, r = (i - 3 + 1) % 3;          /* getCornerNodes (Shape.cpp:455-461) */
    int kl = nd[l], kr = nd[r];
    for( int j=0; j<MAXEQ; j++ ) K[i*MAXEQ+j] = 0.0;
    double Un = m->U[k]*m->niox[k] + m->V[k]*m->nioy[k];
    double Hl = m->S[kl] - m->z[kl];
    double Hr = m->S[kr] - m->z[kr];
    double H = ( Hl + Hr ) / 2.0;
    double specQ = m->bcU[k];
    if( H <= 0.0 ) { H = m->hmin;  specQ = 0.0; }
    f[i] = area * (specQ - Un*H);
    K[i*MAXEQ + i]          = area * H;
    K[i*MAXEQ + eqidS + l]  = area * Un / 2.0;
    K[i*MAXEQ + eqidS + r]  = area * Un / 2.0;
  }
}

int orc_coefs(const orc_model* m, int e, double* K, double* f)
{
  init_shapes();
  int fl = m->eflag[e];
  if( fl & E_DRY ) return 0;
  if( fl & E_BOUND ) coefs_bound( m, e, K, f );
  else               coefs_region( m, e, K, f );
  return 1;
}

/* ------------------------------------------------------------------------ */
/* linear algebra in the two storage precisions                              */

#define REAL float
#define SFX(name) name##_f32
#include "rg_oracle_la.inc"
#undef REAL
#undef SFX

#define REAL double
#define SFX(name) name##_f64
#include "rg_oracle_la.inc"
#undef REAL
#undef SFX

/* ------------------------------------------------------------------------ */
/* Newton correction (EqsUVS2D.cpp:455-759) and friction                     */

void orc_newton_update(const orc_update_cfg* c, const int* eqno, const int* nflag, const double* rot,
                       const double* X, double* U, double* V, double* S, double* z,
                       const double* zor, double hmin, double* stats)
{
  double mx[3] = { 0, 0, 0 };
  double theNorm = 0.0, maxUs = 0.0, maxS = 0.0;
  for( int ii=0; ii<c->np_model; ii++ )
  {
    int n = c->model_nodes[ii];
    for( int v=0; v<3; v++ )
    {
      int q = eqno[3*n+v];
      if( q >= 0 && fabs(X[q]) > mx[v] ) mx[v] = fabs(X[q]);
    }
    double dU = 0, dV = 0, dS = 0;
    if( eqno[3*n+0] >= 0 ) dU = fabs( X[eqno[3*n+0]] );
    if( eqno[3*n+1] >= 0 ) dV = fabs( X[eqno[3*n+1]] );
    if( eqno[3*n+2] >= 0 ) dS = fabs( X[eqno[3*n+2]] );
    theNorm += dU*dU + dV*dV + dS*dS;
    double dUs = sqrt( dU*dU + dV*dV );
    if( dUs > maxUs ) maxUs = dUs;
    if( dS  > maxS  ) maxS  = dS;
  }
  theNorm = sqrt( theNorm );
  double relaxUs = 1.0, relaxS = 1.0;
  if( c->relaxMethod == 2 )
  {
    relaxUs = c->maxDeltaUV / maxUs;
    relaxS  = c->maxDeltaS  / maxS;
    if( relaxUs > 1.0 ) relaxUs = 1.0;
    if( relaxS  > 1.0 ) relaxS  = 1.0;
  }
  int exUV = 0, exS = 0;
  for( int ii=0; ii<c->np_model; ii++ )
  {
    int n = c->model_nodes[ii];
    double dU = 0, dV = 0, dS = 0;
    int qU = eqno[3*n+0], qV = eqno[3*n+1], qS = eqno[3*n+2];
    if( qU >= 0 ) dU = X[qU] * relaxUs;
    if( qV >= 0 ) dV = X[qV] * relaxUs;
    if( qS >= 0 ) dS = X[qS] * relaxS;
    if( nflag[n] & N_ROTAT )
    {
      const double* r = rot + 4*n;
      U[n] += r[0] * dU;
      V[n] += r[2] * dU;
      U[n] += r[1] * dV;
      V[n] += r[3] * dV;
    }
    else
    {
      U[n] += dU;
      V[n] += dV;
    }
    double Uu = U[n], Vv = V[n];
    double Us = sqrt( Uu*Uu + Vv*Vv );
    if( Us > c->maxUs )
    {
      exUV++;
      U[n] = Uu * c->maxUs / Us;
      V[n] = Vv * c->maxUs / Us;
    }
    if( qS >= 0 )
    {
      S[n] += dS;
      if( c->dryRewMethod == 0 || c->dryRewMethod == 2 || c->dryRewMethod == 3 )
      {
        double H = S[n] - zor[n];
        if( H < c->dryLimit ) { exS++;  z[n] = S[n] - c->dryLimit; }
        else                  z[n] = zor[n];
      }
      else
      {
        double H = S[n] - z[n];
        if( H <= 0.0 ) { exS++;  S[n] = z[n] + hmin; }
      }
    }
  }
  for( int e=0; e<c->ne_region; e++ )
  {
    const int* nd = c->region_nodes + 6*e;
    for( int i=3; i<6; i++ )
    {
      int l = nd[i-3], r = nd[(i-3+1)%3];
      S[nd[i]] = 0.5 * ( S[l] + S[r] );
      z[nd[i]] = 0.5 * ( z[l] + z[r] );
    }
  }
  if( stats )
  {
    stats[0] = mx[0];  stats[1] = mx[1];  stats[2] = mx[2];
    stats[3] = relaxUs;  stats[4] = relaxS;  stats[5] = theNorm;
    stats[6] = exUV;  stats[7] = exS;  stats[8] = 0.0;
  }
}

void orc_friction(int np, int ne_region, const int* region_nodes, const int* region_nnd,
                  const double* elem_n, const double* elem_areafact, const double* U,
                  const double* V, const double* S, const double* z, double hmin, double g,
                  double* cf)
{
  int* counter = (int*)calloc( (size_t)np, sizeof(int) );
  for( int i=0; i<np; i++ ) cf[i] = 0.0;
  for( int e=0; e<ne_region; e++ )
  {
    const int* nd = region_nodes + 6*e;
    double rc = elem_n[e];
    for( int i=0; i<region_nnd[e]; i++ )
    {
      int k = nd[i];
      double h = S[k] - z[k];
      if( h < hmin ) h = hmin;
      double c = g * (rc * rc) / pow( h, 0.333333 );
      c += 0.0;    /* Nikuradse form roughness with kd + kr = 0 adds 0 (Friction.cpp:95) */
      cf[k] += elem_areafact[e] * c;
      counter[k]++;
    }
    (void)U; (void)V;
  }
  for( int i=0; i<np; i++ ) if( counter[i] ) cf[i] /= counter[i];
  free( counter );
}


/* MODEL::Continuity (Contin.cpp:83-170): for every control element in order and
 * every Gauss point of the quadratic line (GPdeg 5: 3 points, Shape.cpp:176-177,
 * 220-242; SHAPE::shapeOfLine, Line.cpp:43-160): the unnormalised normal
 * (dN.y, -dN.x), H = M.(S - z) clipped at 0, U and V with the quadratic shape,
 * Qx += w H U nx, Qy += w H V ny (no MPI interfaces here). */
void orc_continuity(int nseg, const int* seg_nodes, const int* seg_section, int nsect, const double* x,
                    const double* y, const double* U, const double* V, const double* S, const double* z,
                    double* Qx, double* Qy)
{
  const double loc[3] = { -sqrt(0.6), 0.0, sqrt(0.6) };
  const double wgt[3] = { 5.0/9.0, 8.0/9.0, 5.0/9.0 };
  for( int i=0; i<nsect; i++ ) Qx[i] = Qy[i] = 0.0;
  for( int e=0; e<nseg; e++ )
  {
    int n = seg_section[e];
    const int* nd = seg_nodes + 3*e;
    for( int g=0; g<3; g++ )
    {
      double xg = loc[g];
      double M[2]  = { (1.0 - xg) / 2.0, (1.0 + xg) / 2.0 };
      double N[3]  = { xg * (xg - 1.0) / 2.0, xg * (xg + 1.0) / 2.0, 1.0 - xg * xg };
      double dN[3] = { xg - 0.5, xg + 0.5, -2.0 * xg };
      double nx =  dN[0]*y[nd[0]] + dN[1]*y[nd[1]] + dN[2]*y[nd[2]];
      double ny = -dN[0]*x[nd[0]] - dN[1]*x[nd[1]] - dN[2]*x[nd[2]];
      double H = M[0] * (S[nd[0]] - z[nd[0]]) + M[1] * (S[nd[1]] - z[nd[1]]);
      if( H <= 0.0 ) H = 0.0;
      double u = N[0]*U[nd[0]] + N[1]*U[nd[1]] + N[2]*U[nd[2]];
      double v = N[0]*V[nd[0]] + N[1]*V[nd[1]] + N[2]*V[nd[2]];
      double w = wgt[g];
      Qx[n-1] += w * H * u * nx;
      Qy[n-1] += w * H * v * ny;
    }
  }
}


int64_t orc_pattern(int np, int ne, const int* enodes, const int* eqno, int neq, int64_t* ptr, int* idx)
{
  /* node -> elements holding it, in element order */
  int64_t* nptr = (int64_t*)calloc( (size_t)np + 1, sizeof(int64_t) );
  for( int e=0; e<ne; e++ )
    for( int i=0; i<6; i++ ) nptr[enodes[6*e+i] + 1]++;
  for( int n=0; n<np; n++ ) nptr[n+1] += nptr[n];
  int* nel = (int*)malloc( (size_t)nptr[np] * sizeof(int) );
  int64_t* fill = (int64_t*)malloc( (size_t)np * sizeof(int64_t) );
  for( int n=0; n<np; n++ ) fill[n] = nptr[n];
  for( int e=0; e<ne; e++ )
    for( int i=0; i<6; i++ ) { int n = enodes[6*e+i]; nel[fill[n]++] = e; }
  int* mark = (int*)malloc( (size_t)np * sizeof(int) );
  for( int n=0; n<np; n++ ) mark[n] = -1;
  int* nb = (int*)malloc( 4096 * sizeof(int) );
  int64_t total;
  for( int eq=0; eq<=neq; eq++ ) ptr[eq] = 0;
  /* pass over nodes: the neighbour list of a node, then one row per equation of the node */
  for( int n=0; n<np; n++ )
  {
    int cnt = 0;
    for( int64_t q=nptr[n]; q<nptr[n+1]; q++ )
    {
      const int* nd = enodes + 6 * nel[q];
      for( int i=0; i<6; i++ )
        if( mark[nd[i]] != n && cnt < 4096 ) { mark[nd[i]] = n; nb[cnt++] = nd[i]; }
    }
    int ncols = 0;
    for( int k=0; k<cnt; k++ )
      for( int v=0; v<3; v++ ) if( eqno[3*nb[k]+v] >= 0 ) ncols++;
    for( int v=0; v<3; v++ )
    {
      int row = eqno[3*n+v];
      if( row < 0 ) continue;
      ptr[row+1] = ncols;
    }
  }
  for( int eq=0; eq<neq; eq++ ) ptr[eq+1] += ptr[eq];
  total = ptr[neq];
  if( idx )
  {
    for( int n=0; n<np; n++ ) mark[n] = -1;
    for( int n=0; n<np; n++ )
    {
      int cnt = 0;
      for( int64_t q=nptr[n]; q<nptr[n+1]; q++ )
      {
        const int* nd = enodes + 6 * nel[q];
        for( int i=0; i<6; i++ )
          if( mark[nd[i]] != n && cnt < 4096 ) { mark[nd[i]] = n; nb[cnt++] = nd[i]; }
      }
      for( int v=0; v<3; v++ )
      {
        int row = eqno[3*n+v];
        if( row < 0 ) continue;
        int64_t o = ptr[row];
        idx[o++] = row;
        for( int k=0; k<cnt; k++ )
          for( int w=0; w<3; w++ )
          {
            int col = eqno[3*nb[k]+w];
            if( col >= 0 && col != row ) idx[o++] = col;
          }
      }
    }
  }
  free( nptr ); free( nel ); free( fill ); free( mark ); free( nb );
  return total;
}
