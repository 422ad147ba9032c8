// mpm_oracle.h — CPU oracle for the implicit MPM snow substep.
//
// TEST INFRASTRUCTURE ONLY. Nothing in the product links, loads or calls this code;
// only the tests, the smoke check and the bench's CPU-baseline leg do, and only as the
// checker (or the timed CPU baseline), never as the thing measured on the GPU.
//
// What it is: a plain C++/OpenMP restatement of the reference's per-substep algorithm
// (SoldierDown/Non_Ficks_Diffusion), templated on the storage type T, the SVD type TS,
// the reduction type TR and the dimension d. Every function cites the reference lines
// it follows.
//
// PARITY UNPINNED against the reference itself: the reference cannot be compiled here
// (it needs the external, un-vendored Nova library) and ships no tests, fixtures or
// golden vectors. This restatement is instead pinned by its own finite-difference and
// known-answer tests (tests/test_oracle_math.py, tests/golden/). Where the reference
// defers to Nova (3x3 SVD, linear solve, conjugate gradient, grid indexing) the oracle
// restates the published algorithm named at each site.
#pragma once
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

// ---------------------------------------------------------------------------------
// Small fixed-size algebra. Matrices are row-major: a[row][col]. The reference's Nova
// matrices store entries column-major; the index formulas below were translated entry
// by entry and are checked by finite differences in the tests.
// ---------------------------------------------------------------------------------
template<class T,int d> struct Vec {
    T v[d];
    Vec(){for(int i=0;i<d;++i) v[i]=T(0);}
    T& operator[](int i){return v[i];}
    const T& operator[](int i) const {return v[i];}
};
template<class T,int d> struct Mat {
    T a[d][d];
    Mat(){for(int i=0;i<d;++i) for(int j=0;j<d;++j) a[i][j]=T(0);}
    static Mat Identity(){Mat m;for(int i=0;i<d;++i) m.a[i][i]=T(1);return m;}
    template<class U> Mat<U,d> cast() const {Mat<U,d> m;for(int i=0;i<d;++i) for(int j=0;j<d;++j) m.a[i][j]=(U)a[i][j];return m;}
};
template<class T,int d> inline Mat<T,d> operator*(const Mat<T,d>& A,const Mat<T,d>& B)
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j){T s=0;for(int k=0;k<d;++k) s+=A.a[i][k]*B.a[k][j];C.a[i][j]=s;}return C;}
template<class T,int d> inline Mat<T,d> Times_Transpose(const Mat<T,d>& A,const Mat<T,d>& B)   // A B^T
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j){T s=0;for(int k=0;k<d;++k) s+=A.a[i][k]*B.a[j][k];C.a[i][j]=s;}return C;}
template<class T,int d> inline Mat<T,d> Transpose_Times(const Mat<T,d>& A,const Mat<T,d>& B)   // A^T B
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j){T s=0;for(int k=0;k<d;++k) s+=A.a[k][i]*B.a[k][j];C.a[i][j]=s;}return C;}
template<class T,int d> inline Mat<T,d> Transpose(const Mat<T,d>& A)
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j) C.a[i][j]=A.a[j][i];return C;}
template<class T,int d> inline Mat<T,d> operator+(const Mat<T,d>& A,const Mat<T,d>& B)
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j) C.a[i][j]=A.a[i][j]+B.a[i][j];return C;}
template<class T,int d> inline Mat<T,d> operator-(const Mat<T,d>& A,const Mat<T,d>& B)
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j) C.a[i][j]=A.a[i][j]-B.a[i][j];return C;}
template<class T,int d> inline Mat<T,d> operator*(const T s,const Mat<T,d>& A)
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j) C.a[i][j]=s*A.a[i][j];return C;}
template<class T,int d> inline Vec<T,d> operator*(const Mat<T,d>& A,const Vec<T,d>& x)
{Vec<T,d> y;for(int i=0;i<d;++i){T s=0;for(int k=0;k<d;++k) s+=A.a[i][k]*x[k];y[i]=s;}return y;}
template<class T,int d> inline Vec<T,d> Transpose_Times(const Mat<T,d>& A,const Vec<T,d>& x)   // A^T x
{Vec<T,d> y;for(int i=0;i<d;++i){T s=0;for(int k=0;k<d;++k) s+=A.a[k][i]*x[k];y[i]=s;}return y;}
template<class T,int d> inline Mat<T,d> Outer_Product(const Vec<T,d>& u,const Vec<T,d>& v)     // u v^T
{Mat<T,d> C;for(int i=0;i<d;++i) for(int j=0;j<d;++j) C.a[i][j]=u[i]*v[j];return C;}
template<class T,int d> inline T Inner(const Mat<T,d>& A,const Mat<T,d>& B)                    // A:B
{T s=0;for(int i=0;i<d;++i) for(int j=0;j<d;++j) s+=A.a[i][j]*B.a[i][j];return s;}

template<class T> inline T Determinant(const Mat<T,2>& A){return A.a[0][0]*A.a[1][1]-A.a[0][1]*A.a[1][0];}
template<class T> inline T Determinant(const Mat<T,3>& A)
{return A.a[0][0]*(A.a[1][1]*A.a[2][2]-A.a[1][2]*A.a[2][1])
       -A.a[0][1]*(A.a[1][0]*A.a[2][2]-A.a[1][2]*A.a[2][0])
       +A.a[0][2]*(A.a[1][0]*A.a[2][1]-A.a[1][1]*A.a[2][0]);}

// Cofactor matrix, cof(F)=det(F) F^{-T} (Nova Matrix::Cofactor_Matrix, used at
// MPM_Constitutive_Model.cpp:50).
template<class T> inline Mat<T,2> Cofactor(const Mat<T,2>& F)
{Mat<T,2> C;C.a[0][0]=F.a[1][1];C.a[0][1]=-F.a[1][0];C.a[1][0]=-F.a[0][1];C.a[1][1]=F.a[0][0];return C;}
template<class T> inline Mat<T,3> Cofactor(const Mat<T,3>& F)
{
    const auto& a=F.a;Mat<T,3> C;
    C.a[0][0]=a[1][1]*a[2][2]-a[1][2]*a[2][1]; C.a[0][1]=a[1][2]*a[2][0]-a[1][0]*a[2][2]; C.a[0][2]=a[1][0]*a[2][1]-a[1][1]*a[2][0];
    C.a[1][0]=a[0][2]*a[2][1]-a[0][1]*a[2][2]; C.a[1][1]=a[0][0]*a[2][2]-a[0][2]*a[2][0]; C.a[1][2]=a[0][1]*a[2][0]-a[0][0]*a[2][1];
    C.a[2][0]=a[0][1]*a[1][2]-a[0][2]*a[1][1]; C.a[2][1]=a[0][2]*a[1][0]-a[0][0]*a[1][2]; C.a[2][2]=a[0][0]*a[1][1]-a[0][1]*a[1][0];
    return C;
}
// Directional derivative of the cofactor matrix: d/de cof(F+e dF).
// MPM_Constitutive_Model.h:28-32 (2D) and :33-46 (3D); product rule on each entry of Cofactor().
template<class T> inline Mat<T,2> Times_Cofactor_Matrix_Derivative(const Mat<T,2>&,const Mat<T,2>& dF)
{return Cofactor(dF);}
template<class T> inline Mat<T,3> Times_Cofactor_Matrix_Derivative(const Mat<T,3>& F,const Mat<T,3>& dF)
{
    const auto& a=F.a; const auto& b=dF.a; Mat<T,3> C;
    auto m=[&](int i,int j,int k,int l){return b[i][j]*a[k][l]+a[i][j]*b[k][l];};
    C.a[0][0]=m(1,1,2,2)-m(1,2,2,1); C.a[0][1]=m(1,2,2,0)-m(1,0,2,2); C.a[0][2]=m(1,0,2,1)-m(1,1,2,0);
    C.a[1][0]=m(0,2,2,1)-m(0,1,2,2); C.a[1][1]=m(0,0,2,2)-m(0,2,2,0); C.a[1][2]=m(0,1,2,0)-m(0,0,2,1);
    C.a[2][0]=m(0,1,1,2)-m(0,2,1,1); C.a[2][1]=m(0,2,1,0)-m(0,0,1,2); C.a[2][2]=m(0,0,1,1)-m(0,1,1,0);
    return C;
}

// ---------------------------------------------------------------------------------
// SVD F = U diag(s) V^T with U, V proper rotations, s[0] >= s[1] >= |s[d-1]| and the sign
// of det(F) carried by the last singular value (the convention of the PhysBAM-lineage
// Fast_Singular_Value_Decomposition that Nova provides, MPM_Constitutive_Model.cpp:36).
// Method: cyclic Jacobi eigen-decomposition of F^T F (Golub & Van Loan, "Matrix
// Computations", sec. 8.5), then U from the columns of F V by Gram-Schmidt and a cross
// product, which keeps U a rotation.
// ---------------------------------------------------------------------------------
template<class T> void SVD(const Mat<T,3>& F,Mat<T,3>& U,Vec<T,3>& s,Mat<T,3>& V)
{
    Mat<T,3> A=Transpose_Times(F,F);
    V=Mat<T,3>::Identity();
    const T eps=std::numeric_limits<T>::epsilon();
    for(int sweep=0;sweep<30;++sweep){
        T off=A.a[0][1]*A.a[0][1]+A.a[0][2]*A.a[0][2]+A.a[1][2]*A.a[1][2];
        T diag=A.a[0][0]*A.a[0][0]+A.a[1][1]*A.a[1][1]+A.a[2][2]*A.a[2][2];
        if(off<=eps*eps*diag*T(1e-2) || off==T(0)) break;
        for(int p=0;p<2;++p) for(int q=p+1;q<3;++q){
            T apq=A.a[p][q];
            if(apq==T(0)) continue;
            T theta=(A.a[q][q]-A.a[p][p])/(T(2)*apq);
            T t=(theta>=T(0)?T(1):T(-1))/(std::fabs(theta)+std::sqrt(theta*theta+T(1)));
            T c=T(1)/std::sqrt(t*t+T(1)),sn=t*c;
            // A <- J^T A J with J the rotation in the (p,q) plane
            for(int k=0;k<3;++k){T akp=A.a[k][p],akq=A.a[k][q];A.a[k][p]=c*akp-sn*akq;A.a[k][q]=sn*akp+c*akq;}
            for(int k=0;k<3;++k){T apk=A.a[p][k],aqk=A.a[q][k];A.a[p][k]=c*apk-sn*aqk;A.a[q][k]=sn*apk+c*aqk;}
            for(int k=0;k<3;++k){T vkp=V.a[k][p],vkq=V.a[k][q];V.a[k][p]=c*vkp-sn*vkq;V.a[k][q]=sn*vkp+c*vkq;}
        }
    }
    // sort eigenvalues descending, permuting V's columns alongside
    T ev[3]={A.a[0][0],A.a[1][1],A.a[2][2]};int idx[3]={0,1,2};
    for(int i=0;i<3;++i) for(int j=i+1;j<3;++j) if(ev[idx[j]]>ev[idx[i]]) std::swap(idx[i],idx[j]);
    Mat<T,3> Vs;for(int k=0;k<3;++k) for(int j=0;j<3;++j) Vs.a[k][j]=V.a[k][idx[j]];
    V=Vs;
    if(Determinant(V)<T(0)) for(int k=0;k<3;++k) V.a[k][2]=-V.a[k][2];
    Mat<T,3> B=F*V;   // columns b_j = F v_j = s_j u_j
    Vec<T,3> b0,b1,b2;for(int k=0;k<3;++k){b0[k]=B.a[k][0];b1[k]=B.a[k][1];b2[k]=B.a[k][2];}
    auto dot=[](const Vec<T,3>& x,const Vec<T,3>& y){return x[0]*y[0]+x[1]*y[1]+x[2]*y[2];};
    auto cross=[](const Vec<T,3>& x,const Vec<T,3>& y){Vec<T,3> z;z[0]=x[1]*y[2]-x[2]*y[1];z[1]=x[2]*y[0]-x[0]*y[2];z[2]=x[0]*y[1]-x[1]*y[0];return z;};
    const T tiny=std::numeric_limits<T>::min()*T(1e4);
    Vec<T,3> u0,u1,u2;
    T n0=std::sqrt(dot(b0,b0));
    if(n0>tiny){for(int k=0;k<3;++k) u0[k]=b0[k]/n0;} else {u0[0]=T(1);}
    T p=dot(u0,b1);for(int k=0;k<3;++k) u1[k]=b1[k]-p*u0[k];
    T n1=std::sqrt(dot(u1,u1));
    if(n1>tiny*T(1e2)*std::max(T(1),n0)){for(int k=0;k<3;++k) u1[k]/=n1;}
    else{ // any unit vector orthogonal to u0
        Vec<T,3> e;int m=0;for(int k=1;k<3;++k) if(std::fabs(u0[k])<std::fabs(u0[m])) m=k;e[m]=T(1);
        T q=dot(u0,e);for(int k=0;k<3;++k) u1[k]=e[k]-q*u0[k];T nn=std::sqrt(dot(u1,u1));for(int k=0;k<3;++k) u1[k]/=nn;}
    u2=cross(u0,u1);
    for(int k=0;k<3;++k){U.a[k][0]=u0[k];U.a[k][1]=u1[k];U.a[k][2]=u2[k];}
    s[0]=dot(u0,b0);s[1]=dot(u1,b1);s[2]=dot(u2,b2);
}
template<class T> void SVD(const Mat<T,2>& F,Mat<T,2>& U,Vec<T,2>& s,Mat<T,2>& V)
{
    Mat<T,2> A=Transpose_Times(F,F);
    V=Mat<T,2>::Identity();
    T apq=A.a[0][1];
    if(apq!=T(0)){
        T theta=(A.a[1][1]-A.a[0][0])/(T(2)*apq);
        T t=(theta>=T(0)?T(1):T(-1))/(std::fabs(theta)+std::sqrt(theta*theta+T(1)));
        T c=T(1)/std::sqrt(t*t+T(1)),sn=t*c;
        T a00=A.a[0][0]-t*apq,a11=A.a[1][1]+t*apq;A.a[0][0]=a00;A.a[1][1]=a11;
        V.a[0][0]=c;V.a[0][1]=sn;V.a[1][0]=-sn;V.a[1][1]=c;}
    if(A.a[1][1]>A.a[0][0]){ // swap columns, keep det(V)=+1
        Mat<T,2> W;W.a[0][0]=V.a[0][1];W.a[1][0]=V.a[1][1];W.a[0][1]=-V.a[0][0];W.a[1][1]=-V.a[1][0];V=W;}
    Mat<T,2> B=F*V;
    T n0=std::sqrt(B.a[0][0]*B.a[0][0]+B.a[1][0]*B.a[1][0]);
    T u0x=T(1),u0y=T(0);
    if(n0>std::numeric_limits<T>::min()*T(1e4)){u0x=B.a[0][0]/n0;u0y=B.a[1][0]/n0;}
    U.a[0][0]=u0x;U.a[1][0]=u0y;U.a[0][1]=-u0y;U.a[1][1]=u0x;
    s[0]=u0x*B.a[0][0]+u0y*B.a[1][0];
    s[1]=-u0y*B.a[0][1]+u0x*B.a[1][1];
}

// Rotation differential dR for the polar rotation R of F (F=R S), given dF.
// MPM_Constitutive_Model.h:47-55 (2D) and :56-69 (3D): R^T dR is the skew matrix W that
// solves W S + S W = M - M^T with M=R^T dF, S=R^T F; in 3D a 3x3 system K (a,b,c)=L
// (Nova Solve_Linear_System, restated here as Cramer's rule with the adjugate).
template<class T> Mat<T,2> dR(const Mat<T,2>& dF,const Mat<T,2>& R,const Mat<T,2>& F)
{
    Mat<T,2> M=Transpose_Times(R,dF),S=Transpose_Times(R,F);
    T a=(M.a[0][1]-M.a[1][0])/(S.a[1][1]+S.a[0][0]);
    Mat<T,2> W;W.a[0][1]=a;W.a[1][0]=-a;
    return R*W;
}
template<class T> Mat<T,3> dR(const Mat<T,3>& dF,const Mat<T,3>& R,const Mat<T,3>& F)
{
    Mat<T,3> M=Transpose_Times(R,dF),S=Transpose_Times(R,F);
    Mat<T,3> K;
    K.a[0][0]=S.a[1][1]+S.a[0][0]; K.a[0][1]=S.a[2][1];            K.a[0][2]=-S.a[2][0];
    K.a[1][0]=S.a[2][1];            K.a[1][1]=S.a[2][2]+S.a[0][0]; K.a[1][2]=S.a[1][0];
    K.a[2][0]=-S.a[2][0];           K.a[2][1]=S.a[1][0];            K.a[2][2]=S.a[2][2]+S.a[1][1];
    Vec<T,3> L;L[0]=M.a[1][0]-M.a[0][1];L[1]=M.a[2][0]-M.a[0][2];L[2]=M.a[2][1]-M.a[1][2];
    Mat<T,3> C=Cofactor(K);T det=Determinant(K);
    Vec<T,3> x=Transpose_Times(C,L);   // adj(K) L = C^T L
    for(int k=0;k<3;++k) x[k]/=det;
    Mat<T,3> W;
    W.a[0][1]=-x[0];W.a[0][2]=-x[1];
    W.a[1][0]= x[0];W.a[1][2]=-x[2];
    W.a[2][0]= x[1];W.a[2][1]= x[2];
    return R*W;
}

// ---------------------------------------------------------------------------------
// Constitutive model: fixed-corotated elasticity with Stomakhin snow plasticity.
// MPM_Constitutive_Model.cpp:23-76. Fp is carried only through Jp=det(Fp), the one
// quantity of Fp that the reference consumes (:48); the update Jp <- Jp*prod(s)/prod(s_hat)
// is det() of the reference's Fp <- V S_hat^-1 U^T Fe Fp.
// ---------------------------------------------------------------------------------
template<class T,int d> struct Constitutive {
    T lambda,mu;   // hardened Lame parameters
    Mat<T,d> Fe,Re,He;T Je;
    Vec<T,d> Se;
    Mat<T,d> P() const   // :63-67
    {return T(2)*mu*(Fe-Re)+(lambda*(Je-T(1)))*He;}
    T Psi() const        // :55-59
    {T s=0;for(int i=0;i<d;++i) s+=(Se[i]-T(1))*(Se[i]-T(1));return mu*s+lambda/T(2)*(Je-T(1))*(Je-T(1));}
    Mat<T,d> Times_dP_dF(const Mat<T,d>& dF) const   // :71-76
    {
        Mat<T,d> dH=Times_Cofactor_Matrix_Derivative(Fe,dF);
        return T(2)*mu*(dF-dR(dF,Re,Fe))+(lambda*Inner(He,dF))*He+(lambda*(Je-T(1)))*dH;
    }
};
// Compute_Lame_Parameters, MPM_Constitutive_Model.cpp:23-28
template<class T> inline void Lame(const T E,const T nu,T& lambda0,T& mu0)
{mu0=E/(T(2)*(T(1)+nu));lambda0=(E*nu)/((T(1)+nu)*(T(1)-T(2)*nu));}

struct PlasticityParams { int plastic; double hardening, compression_yield, stretching_yield, hardening_max; };

// Precompute, MPM_Constitutive_Model.cpp:32-51. The SVD runs in TS; results are rounded to T.
template<class T,class TS,int d>
void Precompute(Mat<T,d>& Fe,T& Jp,const T lambda0,const T mu0,const PlasticityParams& pp,Constitutive<T,d>& cm)
{
    Mat<TS,d> F=Fe.template cast<TS>(),U,V;Vec<TS,d> s;
    SVD(F,U,s,V);
    TS prod_s=1;for(int i=0;i<d;++i) prod_s*=s[i];
    if(pp.plastic){
        const TS sy=(TS)(T)pp.stretching_yield,cy=(TS)(T)pp.compression_yield;
        for(int i=0;i<d;++i) if(s[i]>sy) s[i]=sy;
        for(int i=0;i<d;++i) if(s[i]<cy) s[i]=cy;
        TS prod_hat=1;for(int i=0;i<d;++i) prod_hat*=s[i];
        Jp=(T)((TS)Jp*(prod_s/prod_hat));
        Mat<TS,d> US=U;for(int i=0;i<d;++i) for(int j=0;j<d;++j) US.a[i][j]*=s[j];
        Fe=Times_Transpose(US,V).template cast<T>();
        T power=std::min((T)pp.hardening*(T(1)-Jp),(T)pp.hardening_max);
        cm.lambda=std::exp(power)*lambda0;cm.mu=std::exp(power)*mu0;}
    else{cm.lambda=lambda0;cm.mu=mu0;}
    TS Je=1;for(int i=0;i<d;++i) Je*=s[i];
    cm.Je=(T)Je;
    cm.Re=Times_Transpose(U,V).template cast<T>();
    cm.Fe=Fe;
    cm.He=Cofactor(Fe);
    for(int i=0;i<d;++i) cm.Se[i]=(T)s[i];
}

// ---------------------------------------------------------------------------------
// Quadratic B-spline weights. MPM_Particle.h:79-100 (Update_Weights/Compute_Weights):
// closest cell c = floor(X/dx) on the cell-centred grid over [0,1]^d (Nova Grid; the
// oracle fixes a 0-based origin), x = (X-(center(c)-dx))/dx in [0.5,1.5),
// w0=|.5x^2-1.5x+1.125|, w1=|-(x-1)^2+.75|, w2=|.5(x-2)^2+1.5(x-2)+1.125|,
// dw0=(x-1.5)/dx, dw1=-2(x-1)/dx, dw2=(x-.5)/dx. Node offsets -1..1.
// ---------------------------------------------------------------------------------
template<class T> inline void Compute_Weights(T x,const T one_over_dx,T w[3],T dw[3])
{
    w[0]=std::fabs((T)0.5*x*x-(T)1.5*x+(T)1.125);
    dw[0]=(x-(T)1.5)*one_over_dx;
    x-=(T)1;
    w[1]=std::fabs(-x*x+(T).75);
    dw[1]=(T)(-2)*x*one_over_dx;
    x-=(T)1;
    w[2]=std::fabs((T).5*x*x+(T)1.5*x+(T)1.125);
    dw[2]=(x+(T)1.5)*one_over_dx;
}

struct Barrier { double normal[3]; double surface[3]; double mu; int sticky; };

struct SceneParams {
    int counts[3];
    double gravity[3];
    double flip;
    double cg_abs_tol,cg_rel_tol; int cg_max_iters,cg_min_iters;
    int project;                       // 1: zero CG vectors inside barrier half-spaces
    PlasticityParams plasticity;
    int n_barriers; Barrier barriers[16];
    int eos;                           // 1: every particle is an EOS fluid particle (p.eos)
    double bulk_modulus,eos_gamma;     // MPM_Particle.h:36-37
};

struct StepStats { int cg_iterations; int converged; double cg_residual; double cg_tolerance; long long n_interior; long long n_removed; };

// Cell flags. Nova SPGrid_Flags values are not visible in the reference; these are the
// oracle's own bit assignments for the two flags the path uses.
enum { Flag_Dirichlet=1u, Flag_Interior=2u };

// ---------------------------------------------------------------------------------
// One scene. Methods are named after the MPM_Example methods they restate.
// ---------------------------------------------------------------------------------
template<class T,class TS,class TR,int d>
class MPM_Oracle
{
  public:
    using TV=Vec<T,d>; using TM=Mat<T,d>;
    using scalar=T;
    static constexpr int dim=d;
    SceneParams P;
    int threads;
    T dx[d],one_over_dx[d];
    TV gravity;
    // particle state
    std::vector<TV> X,V; std::vector<TM> Fe; std::vector<T> Jp,mass,V0,lambda0,mu0; std::vector<uint8_t> valid;
    std::vector<int> simulated,waiting;
    // per-substep particle data
    std::vector<int> cc;            // closest cell, d ints per particle
    std::vector<T> w,dw;            // 3*d weights per particle
    std::vector<Constitutive<T,d>> cm;
    std::vector<TM> scp;
    // grid: dense box covering every particle stencil, cells [glo, glo+gn)
    int glo[d],gn[d]; size_t gsize=0;
    int bb_lo[d],bb_hi[d];          // Dirichlet cell range (bounding box, Rasterize_Voxels)
    std::vector<uint32_t> flags;
    std::vector<T> gm; std::vector<TV> gv,gvs,gf,grhs,gr,gs,gq;
    StepStats last;

    explicit MPM_Oracle(const SceneParams& p,int nthreads=0):P(p)
    {
#ifdef _OPENMP
        threads=nthreads>0?nthreads:omp_get_max_threads();
#else
        threads=1;
#endif
        for(int a=0;a<d;++a){dx[a]=T(1)/(T)P.counts[a];one_over_dx[a]=(T)P.counts[a];gravity[a]=(T)P.gravity[a];}
        std::memset(&last,0,sizeof(last));
    }

    void Add_Particle(const T* x,const T* v,T m,T l0,T m0,const T* F,T jp,T v0)
    {
        TV xx,vv;TM FF=TM::Identity();
        for(int a=0;a<d;++a){xx[a]=x[a];vv[a]=v[a];}
        if(F) for(int i=0;i<d;++i) for(int j=0;j<d;++j) FF.a[i][j]=F[i*d+j];
        X.push_back(xx);V.push_back(vv);Fe.push_back(FF);Jp.push_back(jp);mass.push_back(m);V0.push_back(v0);
        lambda0.push_back(l0);mu0.push_back(m0);valid.push_back(1);
    }

    // Allocate_Particle(true), MPM_Example.cpp:959-975: the slot of a removed particle if
    // there is one, else a new particle; the particle is reset (Fe = I, Jp = 1, the
    // reference's Initialize()) and waits for its first-touch volume, which the next
    // substep's Process_Waiting_Particles computes (MPM_Example.cpp:827-840). Slot choice
    // of this build: the removed particle of lowest index (the reference pops the one most
    // recently appended to invalid_particles). Returns the particle's index.
    int Allocate_Particle(const T* x,const T* v,T m,T l0,T m0)
    {
        int id=-1;
        for(size_t i=0;i<X.size();++i) if(!valid[i]){id=(int)i;break;}
        if(id<0){Add_Particle(x,v,m,l0,m0,nullptr,T(1),T(0));id=(int)X.size()-1;}
        else{
            for(int a=0;a<d;++a){X[id][a]=x[a];V[id][a]=v[a];}
            Fe[id]=TM::Identity();Jp[id]=T(1);mass[id]=m;V0[id]=T(0);lambda0[id]=l0;mu0[id]=m0;valid[id]=1;}
        waiting.push_back(id);
        return id;
    }

    // MPM_Example.cpp:347-355
    void Populate_Simulated_Particles()
    {simulated.clear();for(size_t i=0;i<X.size();++i) if(valid[i]) simulated.push_back((int)i);}

    // MPM_Example.cpp:152-161 + MPM_Driver.cpp:18-32 (Initialize): the first grid build and
    // the first-touch volumes.
    void Initialize()
    {
        Populate_Simulated_Particles();
        waiting.clear();for(int id:simulated) if(!(V0[id]>T(0))) waiting.push_back(id);
        Initialize_SPGrid();
        Update_Particle_Weights();
        Rasterize_Voxels();
        Rasterize();
        Process_Waiting_Particles();
    }

    // MPM_Example.cpp:236-265: particle AABB +-2/counts, clamped to [0,1]; the cell range of
    // its corners (Clamp_To_Cell, :298-302) is the Dirichlet-activated set.
    void Compute_Bounding_Box(T bmin[d],T bmax[d])
    {
        for(int a=0;a<d;++a){bmin[a]=T(1);bmax[a]=T(0);}   // domain.max_corner / min_corner
        for(int id:simulated) for(int a=0;a<d;++a){
            const T dd=(T)2./(T)P.counts[a];
            bmin[a]=std::min(bmin[a],X[id][a]-dd);bmax[a]=std::max(bmax[a],X[id][a]+dd);}
        for(int a=0;a<d;++a){bmin[a]=std::max((T)0.,bmin[a]);bmax[a]=std::min((T)1.,bmax[a]);}
    }
    int Clamp_To_Cell(const T x,int a) const
    {int c=(int)std::floor(x*one_over_dx[a]);return std::min(std::max(c,0),P.counts[a]-1);}

    // MPM_Example.cpp:325-331
    void Initialize_SPGrid()
    {
        T bmin[d],bmax[d];Compute_Bounding_Box(bmin,bmax);
        for(int a=0;a<d;++a){bb_lo[a]=Clamp_To_Cell(bmin[a],a);bb_hi[a]=Clamp_To_Cell(bmax[a],a);}
    }

    // MPM_Example.cpp:418-427 and MPM_Particle.h:79-100
    void Update_Particle_Weights()
    {
        const size_t N=X.size();
        cc.assign(N*d,0);w.assign(N*3*d,T(0));dw.assign(N*3*d,T(0));
        const int ns=(int)simulated.size();
#pragma omp parallel for num_threads(threads)
        for(int i=0;i<ns;++i){const int id=simulated[i];
            for(int a=0;a<d;++a){
                const int c=(int)std::floor(X[id][a]*one_over_dx[a]);
                cc[id*d+a]=c;
                const T center=((T)c+(T).5)*dx[a];
                const T xe=X[id][a]-(center-dx[a]);
                Compute_Weights(xe*one_over_dx[a],one_over_dx[a],&w[(id*3)*d+a*3],&dw[(id*3)*d+a*3]);}}
        // dense grid box: the hull of every stencil (cells c-1..c+1)
        int lo[d],hi[d];for(int a=0;a<d;++a){lo[a]=1<<30;hi[a]=-(1<<30);}
        for(int id:simulated) for(int a=0;a<d;++a){lo[a]=std::min(lo[a],cc[id*d+a]-1);hi[a]=std::max(hi[a],cc[id*d+a]+1);}
        gsize=1;for(int a=0;a<d;++a){if(hi[a]<lo[a]){lo[a]=0;hi[a]=0;}glo[a]=lo[a];gn[a]=hi[a]-lo[a]+1;gsize*=(size_t)gn[a];}
    }
    inline T W(int id,int a,int o) const {return w[(id*3)*d+a*3+o];}
    inline T DW(int id,int a,int o) const {return dw[(id*3)*d+a*3+o];}
    inline size_t Node(const int* c) const
    {size_t l=0;for(int a=0;a<d;++a) l=l*(size_t)gn[a]+(size_t)(c[a]-glo[a]);return l;}   // axis 0 slowest
    void Node_Coords(size_t l,int* c) const
    {for(int a=d-1;a>=0;--a){c[a]=(int)(l%(size_t)gn[a])+glo[a];l/=(size_t)gn[a];}}

    // Weight and gradient of stencil offset o (each in 0..2, i.e. node c+o-1):
    // Influence_Iterator.h:85-99
    inline void Stencil(int id,const int* o,T& weight,TV& grad) const
    {
        weight=T(1);for(int a=0;a<d;++a) weight*=W(id,a,o[a]);
        for(int i=0;i<d;++i){T g=T(1);for(int j=0;j<d;++j) g*=(i==j)?DW(id,j,o[j]):W(id,j,o[j]);grad[i]=g;}
    }

    // Race-free scatter: the grid's x range is split into `threads` slabs and each slab
    // walks the particles whose stencil meets it, in increasing particle index, with the
    // stencil cropped to the slab (Group_Particles MPM_Example.cpp:464-485,
    // Cropped_Influence_Iterator.h:31-37). Every node is therefore summed in one fixed order.
    template<class F> void Scatter(F&& f)
    {
        const int T_=std::max(1,std::min(threads,gn[0]));
        const int ns=(int)simulated.size();
#pragma omp parallel for num_threads(T_) schedule(static,1)
        for(int t=0;t<T_;++t){
            const int s_lo=glo[0]+(int)((long long)gn[0]*t/T_),s_hi=glo[0]+(int)((long long)gn[0]*(t+1)/T_)-1;
            for(int i=0;i<ns;++i){const int id=simulated[i];const int c0=cc[id*d];
                if(c0+1<s_lo||c0-1>s_hi) continue;
                const int o0_lo=std::max(0,s_lo-(c0-1)),o0_hi=std::min(2,s_hi-(c0-1));
                f(id,o0_lo,o0_hi);}}
    }
    // Walk the (cropped) stencil, last axis fastest (Influence_Iterator.h:72-76).
    template<class F> inline void Walk(int id,int o0_lo,int o0_hi,F&& f) const
    {
        int o[d],c[d];
        if constexpr(d==2){
            for(o[0]=o0_lo;o[0]<=o0_hi;++o[0]) for(o[1]=0;o[1]<3;++o[1]){
                for(int a=0;a<d;++a) c[a]=cc[id*d+a]+o[a]-1;f(o,Node(c));}}
        else{
            for(o[0]=o0_lo;o[0]<=o0_hi;++o[0]) for(o[1]=0;o[1]<3;++o[1]) for(o[2]=0;o[2]<3;++o[2]){
                for(int a=0;a<d;++a) c[a]=cc[id*d+a]+o[a]-1;f(o,Node(c));}}
    }

    // Rasterize_Voxels (MPM_Example.cpp:291-311) + grid reset (the hierarchy is rebuilt, so
    // every channel starts at zero).
    void Rasterize_Voxels()
    {
        flags.assign(gsize,0u);gm.assign(gsize,T(0));
        gv.assign(gsize,TV());gvs.assign(gsize,TV());gf.assign(gsize,TV());
        grhs.assign(gsize,TV());gr.assign(gsize,TV());gs.assign(gsize,TV());gq.assign(gsize,TV());
        for(size_t l=0;l<gsize;++l){int c[d];Node_Coords(l,c);bool in=true;
            for(int a=0;a<d;++a) if(c[a]<bb_lo[a]||c[a]>bb_hi[a]) in=false;
            if(in) flags[l]|=Flag_Dirichlet;}
    }

    // Rasterize: P2G of m and m v (MPM_Example.cpp:520-537), Flag_Setup_Helper.h:25-35
    // (Interior where m>0), Velocity_Normalization_Helper.h:39-52 (v=mv/m).
    void Rasterize()
    {
        Scatter([&](int id,int lo,int hi){
            Walk(id,lo,hi,[&](const int* o,size_t n){
                T weight;TV g;Stencil(id,o,weight,g);
                const T pm=mass[id];gm[n]+=weight*pm;
                for(int a=0;a<d;++a) gv[n][a]+=weight*(pm*V[id][a]);});});
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l){
            if(gm[l]>T(0)) flags[l]|=Flag_Interior;
            if(flags[l]&Flag_Interior){const T mi=T(1)/gm[l];for(int a=0;a<d;++a) gv[l][a]*=mi;}}
    }

    // MPM_Example.cpp:827-840: V0 = m_p / (sum_i w_ip m_i / dx^d) for particles without a volume.
    void Process_Waiting_Particles()
    {
        T vol=T(1);for(int a=0;a<d;++a) vol*=dx[a];
        const T one_over_volume_per_cell=T(1)/vol;
        const int nw=(int)waiting.size();
#pragma omp parallel for num_threads(threads)
        for(int i=0;i<nw;++i){const int id=waiting[i];T density=T(0);
            Walk(id,0,2,[&](const int* o,size_t n){T weight;TV g;Stencil(id,o,weight,g);density+=weight*gm[n];});
            density*=one_over_volume_per_cell;V0[id]=mass[id]/density;}
        waiting.clear();
    }

    // MPM_Example.cpp:563-571
    void Update_Constitutive_Model_State()
    {
        cm.resize(X.size());scp.resize(X.size());
        const int ns=(int)simulated.size();
#pragma omp parallel for num_threads(threads)
        for(int i=0;i<ns;++i){const int id=simulated[i];
            if(!P.eos) Precompute<T,TS,d>(Fe[id],Jp[id],lambda0[id],mu0[id],P.plasticity,cm[id]);}
    }
    // EOS fluid particles (MPM_Example.cpp:737-738, MPM_CG_System.h:102-107): the explicit
    // force coefficient V0/rho k rho^(gamma-1) and the Hessian coefficient
    // V0 k gamma rho^(gamma-1); rho is the particle density, kept in the Jp slot.
    T Eos_Force_Coefficient(int id) const
    {const T rho=Jp[id];return V0[id]/rho*(T)P.bulk_modulus*(T)std::pow(rho,(T)P.eos_gamma-T(1));}
    T Eos_Hessian_Coefficient(int id) const
    {const T rho=Jp[id];return V0[id]*(T)P.bulk_modulus*(T)P.eos_gamma*(T)std::pow(rho,(T)P.eos_gamma-T(1));}

    // MPM_Example.cpp:757-790 + Explicit_Force_Helper.h:43-56
    void Apply_Explicit_Force(const T dt)
    {
        Scatter([&](int id,int lo,int hi){
            if(P.eos){
                // MPM_Example.cpp:774-783: f += coefficient grad w (no stress term)
                const T coef=Eos_Force_Coefficient(id);
                Walk(id,lo,hi,[&](const int* o,size_t n){
                    T weight;TV g;Stencil(id,o,weight,g);
                    for(int a=0;a<d;++a){const T body=gravity[a]*mass[id]*weight;gf[n][a]+=coef*g[a];gf[n][a]+=body;}});
                return;}
            const T v0=V0[id];const TM V0_P_FT=v0*Times_Transpose(cm[id].P(),Fe[id]);
            Walk(id,lo,hi,[&](const int* o,size_t n){
                T weight;TV g;Stencil(id,o,weight,g);
                TV inner=V0_P_FT*g;
                for(int a=0;a<d;++a){const T body=gravity[a]*mass[id]*weight;gf[n][a]-=inner[a];gf[n][a]+=body;}});});
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior)
            for(int a=0;a<d;++a) gvs[l][a]=gv[l][a]+dt/gm[l]*gf[l][a];
    }

    inline bool Inside_Barrier(const int* c,int b) const
    {
        const Barrier& B=P.barriers[b];T r=T(0);
        for(int a=0;a<d;++a){const T center=((T)c[a]+(T).5)*dx[a];r+=(center-(T)B.surface[a])*(T)B.normal[a];}
        return r<T(0);
    }

    // Grid_Based_Collision_Helper.h:57-85 on v*, barriers in list order. The reference never
    // reads MPM_Plane_Barrier::sticky; here a sticky barrier sets v*=0 inside its half-space.
    void Grid_Based_Collision()
    {
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l){
            if(!(flags[l]&Flag_Interior)) continue;
            int c[d];Node_Coords(l,c);
            for(int b=0;b<P.n_barriers;++b){
                if(!Inside_Barrier(c,b)) continue;
                const Barrier& B=P.barriers[b];
                if(B.sticky){gvs[l]=TV();continue;}
                TV vel=gvs[l],n;for(int a=0;a<d;++a) n[a]=(T)B.normal[a];
                const T mu=(T)B.mu;
                T projection=T(0);for(int a=0;a<d;++a) projection+=vel[a]*n[a];
                if(projection<T(0)){
                    for(int a=0;a<d;++a) vel[a]-=n[a]*projection;
                    T nv=T(0);for(int a=0;a<d;++a) nv+=vel[a]*vel[a];nv=std::sqrt(nv);
                    if(-projection*mu<nv){for(int a=0;a<d;++a) vel[a]+=vel[a]/nv*projection*mu;}
                    else vel=TV();}
                gvs[l]=vel;}}
    }

    // ---- the Krylov system, MPM_CG_System.h:73-249 ----
    // Force (:150-215): pass A gathers dF=(sum_i x_i grad w_i^T) Fe per particle and forms
    // scp = V0 Fe dP^T; pass B scatters f_i += scp^T grad w_i.
    void Force(std::vector<TV>& f,const std::vector<TV>& x)
    {
        const int ns=(int)simulated.size();
#pragma omp parallel for num_threads(threads)
        for(int i=0;i<ns;++i){const int id=simulated[i];TM tmp;
            if(P.eos){
                // MPM_CG_System.h:102-107: eos_scp = coefficient * (sum_i grad w_i . x_i); the
                // scalar is added to a zero matrix, which (as PhysBAM's MATRIX += scalar) puts
                // it on the diagonal, so the scatter below adds eos_scp grad w.
                T div=T(0);
                Walk(id,0,2,[&](const int* o,size_t n){T weight;TV g;Stencil(id,o,weight,g);for(int a=0;a<d;++a) div+=g[a]*x[n][a];});
                const T s=Eos_Hessian_Coefficient(id)*div;
                TM m;for(int a=0;a<d;++a) m.a[a][a]=s;
                scp[id]=m;
                continue;}
            Walk(id,0,2,[&](const int* o,size_t n){T weight;TV g;Stencil(id,o,weight,g);tmp=tmp+Outer_Product(g,x[n]);});
            const TM& F=Fe[id];
            TM dF=Transpose_Times(tmp,F);
            scp[id]=V0[id]*Times_Transpose(F,cm[id].Times_dP_dF(dF));}
        std::fill(f.begin(),f.end(),TV());
        Scatter([&](int id,int lo,int hi){
            Walk(id,lo,hi,[&](const int* o,size_t n){T weight;TV g;Stencil(id,o,weight,g);
                TV t=Transpose_Times(scp[id],g);for(int a=0;a<d;++a) f[n][a]+=t[a];});});
    }
    // Multiply (:73-81) + Multiply_Helper.h:40-53: result = x + dt^2/m * Force(x) on Interior.
    void Multiply(const std::vector<TV>& x,std::vector<TV>& result,const T dt)
    {
        Force(result,x);
        const T scaled_dt_squared=dt*dt;
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior)
            for(int a=0;a<d;++a) result[l][a]=scaled_dt_squared/gm[l]*result[l][a]+x[l][a];
    }
    // Project (:220-225, Project_Helper.h:30-45). The reference's predicate is mis-parenthesised
    // (`Dot_Product(normal<0)`); the oracle implements the intended test, (x-s).n < 0, and
    // zeroes the whole vector there. P.project==0 disables the projection.
    void Project(std::vector<TV>& v)
    {
        if(!P.project||P.n_barriers==0) return;
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l){int c[d];Node_Coords(l,c);
            for(int b=0;b<P.n_barriers;++b) if(Inside_Barrier(c,b)){v[l]=TV();break;}}
    }
    // Inner_Product_Helper.h:45-70: sum over Interior of x . (y m). The per-node term is
    // formed in T and accumulated in TR (FP64 in the mixed and FP64 variants).
    TR Inner_Product(const std::vector<TV>& x,const std::vector<TV>& y)
    {
        TR s=TR(0);
#pragma omp parallel for num_threads(threads) reduction(+:s)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior){
            T t=T(0);for(int a=0;a<d;++a) t+=x[l][a]*(y[l][a]*gm[l]);s+=(TR)t;}
        return s;
    }
    // Convergence_Norm_Helper.h:43-59: max over Interior of |r_i|_2 (|r_i|^2 formed in T).
    TR Convergence_Norm(const std::vector<TV>& r)
    {
        TR m=TR(0);
#pragma omp parallel for num_threads(threads) reduction(max:m)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior){
            T t=T(0);for(int a=0;a<d;++a) t+=r[l][a]*r[l][a];m=std::max(m,(TR)t);}
        return std::sqrt(m);
    }
    // Masked vector update y = a x + y over Interior in T (MPM_CG_Vector.h:90-101, SPGrid
    // Masked_Saxpy); the scalar is rounded to T.
    void Saxpy(const TR a,const std::vector<TV>& x,std::vector<TV>& y)
    {
        const T at=(T)a;
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior)
            for(int k=0;k<d;++k) y[l][k]=at*x[l][k]+y[l][k];
    }

    // Conjugate gradient on the Krylov system. The reference calls Nova's
    // Conjugate_Gradient<T>::Solve (MPM_Example.cpp:702-711), which is not in the reference
    // tree; this restates the PhysBAM-lineage CG it descends from (Hestenes-Stiefel CG,
    // no preconditioner): r=b-Ax, Project(r); loop { stop if Convergence_Norm(r)<=tol
    // (and it>=min or the norm is below epsilon); stop at max; rho=<r,r>; s=r (first) or
    // r+(rho/rho_old)s; q=As; Project(q); alpha=rho/<s,q>; x+=alpha s; r-=alpha q }.
    // The tolerance is max(abs_tol, rel_tol*Convergence_Norm(b)).
    void Solve(const T dt)
    {
        std::vector<TV>& x=gvs;const std::vector<TV>& b=grhs;
        const TR small_number=(TR)std::numeric_limits<T>::epsilon();
        const TR tol=std::max((TR)P.cg_abs_tol,(TR)P.cg_rel_tol*Convergence_Norm(b));
        Multiply(x,gq,dt);
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior) for(int a=0;a<d;++a) gr[l][a]=b[l][a]-gq[l][a];
        Project(gr);
        TR rho_old=(TR)FLT_MAX,cn=0;int it=0;bool converged=false;
        for(it=0;;++it){
            cn=Convergence_Norm(gr);
            if(cn<=tol&&(it>=P.cg_min_iters||cn<small_number)){converged=true;break;}
            if(it>=P.cg_max_iters) break;
            TR rho=Inner_Product(gr,gr);
            if(it==0){
#pragma omp parallel for num_threads(threads)
                for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior) gs[l]=gr[l];}
            else{const T beta=(T)(rho/rho_old);
#pragma omp parallel for num_threads(threads)
                for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior)
                    for(int a=0;a<d;++a) gs[l][a]=gr[l][a]+beta*gs[l][a];}
            Multiply(gs,gq,dt);
            Project(gq);
            TR sq=Inner_Product(gs,gq);
            TR alpha=sq!=TR(0)?rho/sq:(TR)FLT_MAX;
            Saxpy(alpha,gs,x);
            Saxpy(-alpha,gq,gr);
            rho_old=rho;}
        last.cg_iterations=it;last.converged=converged;last.cg_residual=(double)cn;last.cg_tolerance=(double)tol;
    }

    // Apply_Force, MPM_Example.cpp:695-716
    void Apply_Force(const T dt,int stop_after)
    {
        Apply_Explicit_Force(dt);
        Grid_Based_Collision();
        // MPM_RHS_Helper.h:39-50, Reset_Solver_Channels MPM_Example.cpp:191-199
#pragma omp parallel for num_threads(threads)
        for(long long l=0;l<(long long)gsize;++l) if(flags[l]&Flag_Interior) grhs[l]=gvs[l];
        if(stop_after==2) return;
        Solve(dt);
    }

    // Update_Particle_Velocities_And_Positions, MPM_Example.cpp:623-666
    void Update_Particle_Velocities_And_Positions(const T dt,int stop_after=0)
    {
        Apply_Force(dt,stop_after);
        if(stop_after==2||stop_after==3) return;
        const T flip=(T)P.flip;
        T lo[d],hi[d];for(int a=0;a<d;++a){lo[a]=T(0)+(T).5*dx[a];hi[a]=T(1)-(T).5*dx[a];}
        const int ns=(int)simulated.size();
        std::vector<uint8_t> removed(ns,0);
#pragma omp parallel for num_threads(threads)
        for(int i=0;i<ns;++i){const int id=simulated[i];
            TV V_pic,V_flip=V[id];TM grad;
            Walk(id,0,2,[&](const int* o,size_t n){T weight;TV g;Stencil(id,o,weight,g);
                if(weight>T(0)){
                    TV Vg=gvs[n],dV;for(int a=0;a<d;++a) dV[a]=gvs[n][a]-gv[n][a];
                    for(int a=0;a<d;++a){V_pic[a]+=weight*Vg[a];V_flip[a]+=weight*dV[a];}
                    grad=grad+Outer_Product(Vg,g);}});
            if(P.eos){T tr=T(0);for(int a=0;a<d;++a) tr+=grad.a[a][a];Jp[id]/=T(1)+dt*tr;}   // MPM_Example.cpp:646
            else Fe[id]=Fe[id]+(dt*grad)*Fe[id];
            for(int a=0;a<d;++a){V[id][a]=V_flip[a]*flip+V_pic[a]*((T)1.-flip);X[id][a]+=V_pic[a]*dt;}
            bool inside=true;for(int a=0;a<d;++a) if(!(X[id][a]>=lo[a]&&X[id][a]<=hi[a])) inside=false;
            if(!inside){valid[id]=0;removed[i]=1;}}
        long long nr=0;std::vector<int> keep;keep.reserve(ns);
        for(int i=0;i<ns;++i){if(removed[i]) nr++;else keep.push_back(simulated[i]);}
        simulated.swap(keep);last.n_removed=nr;
    }

    // MPM_Driver.cpp:103-116. stop_after: 0 full substep; 1 after Rasterize (m, v, flags);
    // 2 after explicit force and collision (v*); 3 after the CG solve.
    void Advance_Step(const T dt,int stop_after=0)
    {
        Populate_Simulated_Particles();
        Initialize_SPGrid();
        Update_Particle_Weights();
        Rasterize_Voxels();
        Rasterize();
        Process_Waiting_Particles();
        last.n_interior=0;for(size_t l=0;l<gsize;++l) if(flags[l]&Flag_Interior) last.n_interior++;
        if(stop_after==1) return;
        Update_Constitutive_Model_State();
        Update_Particle_Velocities_And_Positions(dt,stop_after);
    }

    // MPM_Example.cpp:375-387
    T Max_Particle_Velocity() const
    {T r=T(0);for(size_t i=0;i<X.size();++i) if(valid[i]){T s=0;for(int a=0;a<d;++a) s+=V[i][a]*V[i][a];r=std::max(r,s);}return std::sqrt(r);}

    // Flag_Helper.h:31-60 counts over the activated set: Dirichlet (every cell of the
    // bounding box is activated, MPM_Example.cpp:298-302), Interior, both. The dense box of
    // this oracle covers only the stencils, so the Dirichlet count is the box's cell count.
    void Flag_Counts(long long out[3]) const
    {
        out[0]=1;for(int a=0;a<d;++a) out[0]*=(long long)(bb_hi[a]-bb_lo[a]+1);
        out[1]=out[2]=0;
        for(size_t l=0;l<gsize;++l){const uint32_t f=flags[l];
            if(f&Flag_Interior) out[1]++;if((f&Flag_Dirichlet)&&(f&Flag_Interior)) out[2]++;}}
};

} // namespace oracle
