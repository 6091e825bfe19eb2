// Dump hooks linked into the reference solver through -Wl,--wrap (oracle/Makefile).
//
// Test infrastructure only.  The hooks do not change what the reference computes;
// they record, for every Newton iteration of EQS_UVS2D::Execute, the inputs and
// outputs of the hot path so that the golden-fixture generator can pin both the
// oracle restatement and the GPU library:
//
//   STATE  node / element / boundary data handed to CRSMAT::AssembleEqs_im
//          (Assemble.cpp:195) -- the element kernels' complete input
//   CRS    the CRS pattern and assembled (unscaled) float values, plus B
//          (Assemble.cpp:195-343 output)
//   SCALE  ||B||_2 returned by CRSMAT::ScaleL2Norm (CRSMat.cpp:319)
//   X      the correction returned by EQS::Solve (Solve.cpp:53) and the
//          BiCGStab iteration count
//   FINAL  node state after EQS_UVS2D::Execute returns (one time step)
//
// Records are written to the file named by $RG_DUMP (nothing is written when it
// is unset): an 8-byte tag, an int64 payload size, the payload.
//
// With $RG_DUMP_LIGHT=1 (large meshes) only small records are written:
//   SCALE  as above
//   XL     solver status, BiCGStab count and the wall time of EQS::Solve
//   ASML   wall time of the assembly
//   FINALL wall time of the whole time step, then per node U, V, S, z and flag

#define protected public
#define private public
#include "Defs.h"
#include "Report.h"
#include "Node.h"
#include "Elem.h"
#include "Model.h"
#include "Grid.h"
#include "Project.h"
#include "Type.h"
#include "CRSMat.h"
#include "Eqs.h"
#include "EqsUVS2D.h"
#include "Solver.h"
#undef protected
#undef private

#include <vector>
#include <string>
#include <stdint.h>

static FILE* dump_file()
{
  static FILE* f = NULL;
  static int opened = 0;
  if( !opened )
  {
    opened = 1;
    const char* p = getenv( "RG_DUMP" );
    if( p && *p )  f = fopen( p, "wb" );
  }
  return f;
}

struct Rec
{
  std::vector<char> buf;
  template<class T> void put( const T& v ) { const char* p = (const char*)&v; buf.insert( buf.end(), p, p + sizeof(T) ); }
  template<class T> void arr( const std::vector<T>& v )
  {
    int64_t n = (int64_t)v.size();
    put( n );
    const char* p = (const char*)v.data();
    buf.insert( buf.end(), p, p + n * sizeof(T) );
  }
  void write( const char* tag )
  {
    FILE* f = dump_file();
    if( !f ) return;
    char t[8] = {0};
    strncpy( t, tag, 8 );
    int64_t n = (int64_t)buf.size();
    fwrite( t, 1, 8, f );
    fwrite( &n, sizeof(n), 1, f );
    fwrite( buf.data(), 1, buf.size(), f );
    fflush( f );
  }
};

static EQS_UVS2D* g_eqs = NULL;    // equation object of the running Newton step

static int light_mode()
{
  static int m = -1;
  if( m < 0 )
  {
    const char* p = getenv( "RG_DUMP_LIGHT" );
    m = ( p && *p == '1' ) ? 1 : 0;
  }
  return m;
}

#include <time.h>
static double wall_s()
{
  struct timespec ts;
  clock_gettime( CLOCK_MONOTONIC, &ts );
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

static void dump_final_light( double seconds, MODEL* model )
{
  GRID* rg = model->region;
  int np = rg->Getnp();
  Rec r;
  std::vector<double> U, V, S, z;
  std::vector<int> flag;
  for( int n=0; n<np; n++ )
  {
    NODE* nd = rg->Getnode(n);
    U.push_back( nd->v.U );  V.push_back( nd->v.V );  S.push_back( nd->v.S );
    z.push_back( nd->z );    flag.push_back( nd->flag );
  }
  r.put( seconds );
  r.put( (int32_t)np );
  r.arr( U ); r.arr( V ); r.arr( S ); r.arr( z ); r.arr( flag );
  r.write( "FINALL" );
}

static void dump_state( const char* tag, EQS* eqs, MODEL* model, PROJECT* project )
{
  GRID* rg = model->region;
  int np = rg->Getnp();

  Rec r;
  std::vector<int> ino, iname, iflag, ibckind, irot, eq0, eq1, eq2, icd;
  std::vector<double> x, y, z, zor, U, V, S, dUdt, dVdt, dSdt, cf, cfw, vt, uu, uv, vv,
                      oU, oV, oS, odUdt, odVdt, odSdt,
                      r00, r01, r10, r11, niox, nioy, nx, ny, bcU, bcV, bcS, bcQ, bcA;

  for( int n=0; n<np; n++ )
  {
    NODE* nd = rg->Getnode(n);
    ino.push_back( nd->Getno() );
    iname.push_back( nd->Getname() );
    iflag.push_back( nd->flag );
    ibckind.push_back( nd->bc.kind );
    irot.push_back( nd->bc.rot );
    icd.push_back( nd->countDown );
    x.push_back( nd->x );  y.push_back( nd->y );
    z.push_back( nd->z );  zor.push_back( nd->zor );
    U.push_back( nd->v.U );  V.push_back( nd->v.V );  S.push_back( nd->v.S );
    dUdt.push_back( nd->v.dUdt );  dVdt.push_back( nd->v.dVdt );  dSdt.push_back( nd->v.dSdt );
    oU.push_back( nd->vo.U );  oV.push_back( nd->vo.V );  oS.push_back( nd->vo.S );
    odUdt.push_back( nd->vo.dUdt );  odVdt.push_back( nd->vo.dVdt );  odSdt.push_back( nd->vo.dSdt );
    cf.push_back( nd->cf );  cfw.push_back( nd->cfw );  vt.push_back( nd->vt );
    uu.push_back( nd->uu );  uv.push_back( nd->uv );  vv.push_back( nd->vv );
    r00.push_back( nd->bc.Getrot(0,0) );  r01.push_back( nd->bc.Getrot(0,1) );
    r10.push_back( nd->bc.Getrot(1,0) );  r11.push_back( nd->bc.Getrot(1,1) );
    niox.push_back( nd->bc.niox );  nioy.push_back( nd->bc.nioy );
    nx.push_back( nd->bc.nx );  ny.push_back( nd->bc.ny );
    bcU.push_back( nd->bc.val ? nd->bc.val->U : 0.0 );
    bcV.push_back( nd->bc.val ? nd->bc.val->V : 0.0 );
    bcS.push_back( nd->bc.val ? nd->bc.val->S : 0.0 );
    bcQ.push_back( nd->bc.val ? nd->bc.val->Q : 0.0 );
    bcA.push_back( nd->bc.val ? nd->bc.val->A : 0.0 );
    if( eqs && eqs->nodeEqno )
    {
      eq0.push_back( eqs->nodeEqno[0][nd->Getno()] );
      eq1.push_back( eqs->nodeEqno[1][nd->Getno()] );
      eq2.push_back( eqs->nodeEqno[2][nd->Getno()] );
    }
    else
    {
      eq0.push_back( -1 );  eq1.push_back( -1 );  eq2.push_back( -1 );
    }
  }

  r.put( (int32_t)np );
  r.arr( ino ); r.arr( iname ); r.arr( iflag ); r.arr( ibckind ); r.arr( irot ); r.arr( icd );
  r.arr( x ); r.arr( y ); r.arr( z ); r.arr( zor );
  r.arr( U ); r.arr( V ); r.arr( S ); r.arr( dUdt ); r.arr( dVdt ); r.arr( dSdt );
  r.arr( oU ); r.arr( oV ); r.arr( oS ); r.arr( odUdt ); r.arr( odVdt ); r.arr( odSdt );
  r.arr( cf ); r.arr( cfw ); r.arr( vt ); r.arr( uu ); r.arr( uv ); r.arr( vv );
  r.arr( r00 ); r.arr( r01 ); r.arr( r10 ); r.arr( r11 );
  r.arr( niox ); r.arr( nioy ); r.arr( nx ); r.arr( ny );
  r.arr( bcU ); r.arr( bcV ); r.arr( bcS ); r.arr( bcQ ); r.arr( bcA );
  r.arr( eq0 ); r.arr( eq1 ); r.arr( eq2 );

  // model element list: region elements followed by their boundary line elements
  std::vector<int> eflag, etype, ennd, ename, enodes, eregion;
  std::vector<double> earea;
  for( int e=0; e<model->ne; e++ )
  {
    ELEM* el = model->elem[e];
    eflag.push_back( el->flag );
    etype.push_back( el->type );
    ennd.push_back( el->Getnnd() );
    ename.push_back( el->Getname() );
    earea.push_back( el->areaFact );
    for( int i=0; i<6; i++ )
      enodes.push_back( i < el->Getnnd() ? el->nd[i]->Getno() : -1 );
  }
  r.arr( eflag ); r.arr( etype ); r.arr( ennd ); r.arr( ename ); r.arr( earea ); r.arr( enodes );

  // all region elements (including dry ones) with their flags and area factors
  std::vector<int> rflag, rnodes, rtype;
  std::vector<double> rarea;
  for( int e=0; e<rg->Getne(); e++ )
  {
    ELEM* el = rg->Getelem(e);
    rflag.push_back( el->flag );
    rtype.push_back( el->type );
    rarea.push_back( el->areaFact );
    for( int i=0; i<6; i++ )
      rnodes.push_back( i < el->Getnnd() ? el->nd[i]->Getno() : -1 );
  }
  r.arr( rflag ); r.arr( rtype ); r.arr( rarea ); r.arr( rnodes );

  // wet node list
  std::vector<int> mnodes;
  for( int n=0; n<model->np; n++ )  mnodes.push_back( model->node[n]->Getno() );
  r.arr( mnodes );

  // scalars
  std::vector<double> sc;
  EQS_UVS2D* ue = g_eqs;
  sc.push_back( ue ? ue->relaxThdt_UV : 0.0 );
  sc.push_back( ue ? ue->relaxThdt_H  : 0.0 );
  sc.push_back( project->g );
  sc.push_back( project->hmin );
  sc.push_back( project->vk );
  sc.push_back( (double)project->actualTurb );
  sc.push_back( (double)project->actualDisp );
  sc.push_back( (double)(eqs ? eqs->neq : 0) );
  sc.push_back( project->timeint.actualTime.Getsec() );
  sc.push_back( project->timeint.incTime.Getsec() );
  sc.push_back( (double)project->GetTimeStep() );
  r.arr( sc );

  // material table: (no, rtype, rcoef, vt)
  std::vector<double> mt;
  for( int t=0; t<TYPE::nType; t++ )
  {
    TYPE* ty = &TYPE::pType[t];
    mt.push_back( (double)ty->_no );
    mt.push_back( (double)ty->rtype );
    mt.push_back( ty->rcoef );
    mt.push_back( ty->vt );
  }
  r.arr( mt );

  r.write( tag );
}


extern "C" {

void   __real__ZN6CRSMAT14AssembleEqs_imEP3EQSPdP5MODELP7PROJECT( CRSMAT*, EQS*, double*, MODEL*, PROJECT* );
double __real__ZN6CRSMAT11ScaleL2NormEPdP6SUBDOM( CRSMAT*, double*, SUBDOM* );
int    __real__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi( EQS*, MODEL*, int, double*, double*,
                                                                    PROJECT*, SOLVER*, PRECON**, int );
void   __real__ZN9EQS_UVS2D7ExecuteEP7PROJECTi( EQS_UVS2D*, PROJECT*, int );


void __wrap__ZN6CRSMAT14AssembleEqs_imEP3EQSPdP5MODELP7PROJECT( CRSMAT* crs, EQS* eqs, double* vec,
                                                               MODEL* model, PROJECT* project )
{
  if( light_mode() )
  {
    double t0 = wall_s();
    __real__ZN6CRSMAT14AssembleEqs_imEP3EQSPdP5MODELP7PROJECT( crs, eqs, vec, model, project );
    Rec r;
    r.put( wall_s() - t0 );
    r.put( (int32_t)crs->m_neq );
    r.write( "ASML" );
    return;
  }
  dump_state( "STATE", eqs, model, project );

  __real__ZN6CRSMAT14AssembleEqs_imEP3EQSPdP5MODELP7PROJECT( crs, eqs, vec, model, project );

  Rec r;
  int neq = crs->m_neq;
  std::vector<int> width( crs->m_width, crs->m_width + neq ), index;
  std::vector<float> A;
  std::vector<double> B( vec, vec + neq );
  for( int i=0; i<neq; i++ )
  {
    for( int j=0; j<crs->m_width[i]; j++ )
    {
      index.push_back( crs->m_index[i][j] );
      A.push_back( (float)crs->m_A[i][j] );
    }
  }
  r.put( (int32_t)neq );
  r.arr( width ); r.arr( index ); r.arr( A ); r.arr( B );
  r.write( "CRS" );
}

double __wrap__ZN6CRSMAT11ScaleL2NormEPdP6SUBDOM( CRSMAT* crs, double* b, SUBDOM* sd )
{
  double s = __real__ZN6CRSMAT11ScaleL2NormEPdP6SUBDOM( crs, b, sd );
  Rec r;
  r.put( s );
  r.write( "SCALE" );
  return s;
}

int __wrap__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi( EQS* eqs, MODEL* model, int neq,
                                                                  double* B, double* X, PROJECT* project,
                                                                  SOLVER* slv, PRECON** pre, int assemble )
{
  double t0 = wall_s();
  int err = __real__ZN3EQS5SolveEP5MODELiPdS2_P7PROJECTP6SOLVERPP6PRECONi( eqs, model, neq, B, X, project,
                                                                          slv, pre, assemble );
  SOLVER* s = slv ? slv : project->actualSolver;
  Rec r;
  if( light_mode() )
  {
    r.put( (int32_t)err );
    r.put( (int32_t)(s ? s->iterCountCG : -1) );
    r.put( wall_s() - t0 );
    r.write( "XL" );
    return err;
  }
  std::vector<double> x( X, X + neq );
  r.put( (int32_t)err );
  r.put( (int32_t)(s ? s->iterCountCG : -1) );
  r.arr( x );
  r.write( "X" );
  return err;
}

void __wrap__ZN9EQS_UVS2D7ExecuteEP7PROJECTi( EQS_UVS2D* eqs, PROJECT* project, int steady )
{
  g_eqs = eqs;
  double t0 = wall_s();
  __real__ZN9EQS_UVS2D7ExecuteEP7PROJECTi( eqs, project, steady );
  if( light_mode() )
    dump_final_light( wall_s() - t0, project->M2D );
  else
    dump_state( "FINAL", eqs, project->M2D, project );
  g_eqs = NULL;
}

}
