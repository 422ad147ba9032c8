// mpm_math.cuh — precision policies and per-particle 3x3 algebra for the sm_103a kernels:
// quadratic B-spline weights, a 3x3 SVD, fixed-corotated stress, its differential and the
// Stomakhin snow-plasticity clamp. Matrices are row-major arrays a[3*i+j].
#pragma once
#include <cuda_runtime.h>
#include <cstdint>
#include <cfloat>

#define MPM_HD __host__ __device__ __forceinline__

namespace mpm {

// T: particle/grid storage and transfer arithmetic. TS: SVD/polar arithmetic. TR: CG dot
// products and norms (per-thread accumulation; cross-thread sums are FP64 in every mode).
// xfer_blocks: resident CTAs per SM the transfer kernels are compiled for (register cap).
struct PrecFP32  { using T=float;  using TS=float;  using TR=float;  static constexpr int id=0; static constexpr int xfer_blocks=4; };
struct PrecMixed { using T=float;  using TS=double; using TR=double; static constexpr int id=1; static constexpr int xfer_blocks=4; };
struct PrecFP64  { using T=double; using TS=double; using TR=double; static constexpr int id=2; static constexpr int xfer_blocks=2; };

template<class T> struct Vec4 { T x,y,z,w; };
template<> struct Vec4<float> { float x,y,z,w; };

template<class T> MPM_HD T mpm_sqrt(T x);
template<> MPM_HD float mpm_sqrt<float>(float x){return sqrtf(x);}
template<> MPM_HD double mpm_sqrt<double>(double x){return sqrt(x);}
template<class T> MPM_HD T mpm_abs(T x){return x<T(0)?-x:x;}
template<class T> MPM_HD T mpm_exp(T x);
template<> MPM_HD float mpm_exp<float>(float x){return expf(x);}
template<> MPM_HD double mpm_exp<double>(double x){return exp(x);}

// ---- 3x3 helpers (row-major) ----
template<class T> MPM_HD void mat_mul(const T* A,const T* B,T* C)          // C = A B
{
#pragma unroll
    for(int i=0;i<3;++i)
#pragma unroll
        for(int j=0;j<3;++j) C[3*i+j]=A[3*i]*B[j]+A[3*i+1]*B[3+j]+A[3*i+2]*B[6+j];
}
template<class T> MPM_HD void mat_mul_bt(const T* A,const T* B,T* C)       // C = A B^T
{
#pragma unroll
    for(int i=0;i<3;++i)
#pragma unroll
        for(int j=0;j<3;++j) C[3*i+j]=A[3*i]*B[3*j]+A[3*i+1]*B[3*j+1]+A[3*i+2]*B[3*j+2];
}
template<class T> MPM_HD void mat_mul_at(const T* A,const T* B,T* C)       // C = A^T B
{
#pragma unroll
    for(int i=0;i<3;++i)
#pragma unroll
        for(int j=0;j<3;++j) C[3*i+j]=A[i]*B[j]+A[3+i]*B[3+j]+A[6+i]*B[6+j];
}
template<class T> MPM_HD T det3(const T* a)
{return a[0]*(a[4]*a[8]-a[5]*a[7])-a[1]*(a[3]*a[8]-a[5]*a[6])+a[2]*(a[3]*a[7]-a[4]*a[6]);}
template<class T> MPM_HD void cofactor3(const T* a,T* C)                   // det(F) F^{-T}
{
    C[0]=a[4]*a[8]-a[5]*a[7]; C[1]=a[5]*a[6]-a[3]*a[8]; C[2]=a[3]*a[7]-a[4]*a[6];
    C[3]=a[2]*a[7]-a[1]*a[8]; C[4]=a[0]*a[8]-a[2]*a[6]; C[5]=a[1]*a[6]-a[0]*a[7];
    C[6]=a[1]*a[5]-a[2]*a[4]; C[7]=a[2]*a[3]-a[0]*a[5]; C[8]=a[0]*a[4]-a[1]*a[3];
}
// d/de cof(F + e dF): product rule on each cofactor entry (reference
// MPM_Constitutive_Model.h:33-46).
template<class T> MPM_HD void cofactor3_diff(const T* a,const T* b,T* C)
{
    C[0]=b[4]*a[8]+a[4]*b[8]-b[5]*a[7]-a[5]*b[7];
    C[1]=b[5]*a[6]+a[5]*b[6]-b[3]*a[8]-a[3]*b[8];
    C[2]=b[3]*a[7]+a[3]*b[7]-b[4]*a[6]-a[4]*b[6];
    C[3]=b[2]*a[7]+a[2]*b[7]-b[1]*a[8]-a[1]*b[8];
    C[4]=b[0]*a[8]+a[0]*b[8]-b[2]*a[6]-a[2]*b[6];
    C[5]=b[1]*a[6]+a[1]*b[6]-b[0]*a[7]-a[0]*b[7];
    C[6]=b[1]*a[5]+a[1]*b[5]-b[2]*a[4]-a[2]*b[4];
    C[7]=b[2]*a[3]+a[2]*b[3]-b[0]*a[5]-a[0]*b[5];
    C[8]=b[0]*a[4]+a[0]*b[4]-b[1]*a[3]-a[1]*b[3];
}

// ---- quadratic B-spline weights (reference MPM_Particle.h:79-100) ----
// x = (X - (center(c) - dx))/dx in [0.5, 1.5); weights of nodes c-1, c, c+1 and their
// derivatives. Products and sums are rounded separately (no contraction) so the weight
// set, and with it the Interior node set, is the same on every machine.
template<class T> MPM_HD void bspline_weights(T x,const T inv_dx,T w[3],T dw[3]);
template<> MPM_HD void bspline_weights<float>(float x,const float inv_dx,float w[3],float dw[3])
{
#ifdef __CUDA_ARCH__
    w[0]=fabsf(__fadd_rn(__fsub_rn(__fmul_rn(__fmul_rn(0.5f,x),x),__fmul_rn(1.5f,x)),1.125f));
    dw[0]=__fmul_rn(__fsub_rn(x,1.5f),inv_dx);
    float y=__fsub_rn(x,1.f);
    w[1]=fabsf(__fadd_rn(-__fmul_rn(y,y),.75f));
    dw[1]=__fmul_rn(__fmul_rn(-2.f,y),inv_dx);
    y=__fsub_rn(y,1.f);
    w[2]=fabsf(__fadd_rn(__fadd_rn(__fmul_rn(__fmul_rn(.5f,y),y),__fmul_rn(1.5f,y)),1.125f));
    dw[2]=__fmul_rn(__fadd_rn(y,1.5f),inv_dx);
#else
    w[0]=fabsf(0.5f*x*x-1.5f*x+1.125f); dw[0]=(x-1.5f)*inv_dx;
    float y=x-1.f; w[1]=fabsf(-y*y+.75f); dw[1]=-2.f*y*inv_dx;
    y-=1.f; w[2]=fabsf(.5f*y*y+1.5f*y+1.125f); dw[2]=(y+1.5f)*inv_dx;
#endif
}
template<> MPM_HD void bspline_weights<double>(double x,const double inv_dx,double w[3],double dw[3])
{
#ifdef __CUDA_ARCH__
    w[0]=fabs(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(0.5,x),x),-__dmul_rn(1.5,x)),1.125));
    dw[0]=__dmul_rn(__dadd_rn(x,-1.5),inv_dx);
    double y=__dadd_rn(x,-1.);
    w[1]=fabs(__dadd_rn(-__dmul_rn(y,y),.75));
    dw[1]=__dmul_rn(__dmul_rn(-2.,y),inv_dx);
    y=__dadd_rn(y,-1.);
    w[2]=fabs(__dadd_rn(__dadd_rn(__dmul_rn(__dmul_rn(.5,y),y),__dmul_rn(1.5,y)),1.125));
    dw[2]=__dmul_rn(__dadd_rn(y,1.5),inv_dx);
#else
    w[0]=fabs(0.5*x*x-1.5*x+1.125); dw[0]=(x-1.5)*inv_dx;
    double y=x-1.; w[1]=fabs(-y*y+.75); dw[1]=-2.*y*inv_dx;
    y-=1.; w[2]=fabs(.5*y*y+1.5*y+1.125); dw[2]=(y+1.5)*inv_dx;
#endif
}

// ---- 3x3 SVD ----
// F = U diag(s) V^T, U and V rotations, s0 >= s1 >= |s2|, sign of det F on s2 (the
// convention of the Fast_Singular_Value_Decomposition the reference calls,
// MPM_Constitutive_Model.cpp:36). Cyclic Jacobi on the symmetric F^T F (Golub & Van
// Loan, "Matrix Computations", sec. 8.5) with at most `max_sweeps` sweeps, then U from the
// columns of F V by Gram-Schmidt and a cross product.
// With a warm start `V0` (orthonormal columns, e.g. the FP32 solution of the same F) the
// sweeps start from A = V0^T F^T F V0, which is already nearly diagonal. The sweeps stop
// once the off-diagonal mass is below (rel |diag|)^2; rel <= 0 means the epsilon of T.
template<class T,int max_sweeps=6> MPM_HD void svd3(const T* F,T* U,T* s,T* V,const T* V0=nullptr,T rel=T(0))
{
    T v[9]={T(1),T(0),T(0),T(0),T(1),T(0),T(0),T(0),T(1)};
    // A = F^T F, or with a warm start V0^T F^T F V0 = B^T B with B = F V0 (the column dot
    // products of B: 45 multiply-adds instead of 72 through F^T F)
    const T* C=F;
    T B0[9];
    if(V0){
#pragma unroll
        for(int k=0;k<9;++k) v[k]=V0[k];
        mat_mul(F,v,B0);C=B0;}
    T a00=C[0]*C[0]+C[3]*C[3]+C[6]*C[6];
    T a01=C[0]*C[1]+C[3]*C[4]+C[6]*C[7];
    T a02=C[0]*C[2]+C[3]*C[5]+C[6]*C[8];
    T a11=C[1]*C[1]+C[4]*C[4]+C[7]*C[7];
    T a12=C[1]*C[2]+C[4]*C[5]+C[7]*C[8];
    T a22=C[2]*C[2]+C[5]*C[5]+C[8]*C[8];
    const T eps=rel>T(0)?rel:(sizeof(T)==4?T(1.1920929e-7):T(2.220446049250313e-16));
    auto rotate=[&](T& app,T& aqq,T& apq,T& arp,T& arq,int p,int q){
        if(apq==T(0)) return;
        // t = tan of the rotation angle = sgn(theta)/(|theta| + sqrt(theta^2 + 1)) with
        // theta = (aqq - app)/(2 apq). Near the diagonal (warm starts, late sweeps) r =
        // 1/(2 theta) is small and t = 2r/(1 + sqrt(1 + 4r^2)) = r(1 - r^2 + 2r^4) + O(r^7),
        // c = (1 + t^2)^(-1/2) = 1 - t^2/2 + 3t^4/8 + O(t^6): relative errors below 1e-23
        // for |r| <= 1e-4, with one division instead of three divisions and two roots.
        const T d=aqq-app;
        T t,c;
        if(mpm_abs(apq)<=T(1e-4)*mpm_abs(d)){
            const T r=apq/d,r2=r*r;
            t=r*(T(1)-r2+T(2)*r2*r2);
            const T t2=t*t;
            c=T(1)-t2*(T(0.5)-T(0.375)*t2);}
        else{
            const T theta=d/(T(2)*apq);
            t=(theta>=T(0)?T(1):T(-1))/(mpm_abs(theta)+mpm_sqrt(theta*theta+T(1)));
            c=T(1)/mpm_sqrt(t*t+T(1));}
        const T sn=t*c;
        app-=t*apq; aqq+=t*apq; apq=T(0);
        T rp=arp,rq=arq; arp=c*rp-sn*rq; arq=sn*rp+c*rq;    // the remaining off-diagonal pair
#pragma unroll
        for(int k=0;k<3;++k){T vp=v[3*k+p],vq=v[3*k+q];v[3*k+p]=c*vp-sn*vq;v[3*k+q]=sn*vp+c*vq;}
    };
#pragma unroll 1
    for(int sweep=0;sweep<max_sweeps;++sweep){
        // off-diagonal mass below (eps |diag|)^2: further rotations only move rounding noise
        T off=a01*a01+a02*a02+a12*a12,diag=a00*a00+a11*a11+a22*a22;
        if(off<=eps*eps*diag) break;
        rotate(a00,a11,a01,a02,a12,0,1);   // (p,q)=(0,1): the other pair is (a02,a12)
        rotate(a00,a22,a02,a01,a12,0,2);   // (0,2): (a01,a21)
        rotate(a11,a22,a12,a01,a02,1,2);   // (1,2): (a10,a20)
    }
    // sort the eigenvalues of F^T F descending with V's columns
    T e0=a00,e1=a11,e2=a22;
    auto swapc=[&](int i,int j){
#pragma unroll
        for(int k=0;k<3;++k){T t=v[3*k+i];v[3*k+i]=v[3*k+j];v[3*k+j]=t;}};
    if(e1>e0){T t=e0;e0=e1;e1=t;swapc(0,1);}
    if(e2>e0){T t=e0;e0=e2;e2=t;swapc(0,2);}
    if(e2>e1){T t=e1;e1=e2;e2=t;swapc(1,2);}
    if(det3(v)<T(0)){v[2]=-v[2];v[5]=-v[5];v[8]=-v[8];}
    T B[9];mat_mul(F,v,B);
    T b0[3]={B[0],B[3],B[6]},b1[3]={B[1],B[4],B[7]},b2[3]={B[2],B[5],B[8]};
    const T tiny=sizeof(T)==4?T(1e-30):T(1e-290);
    T n0=mpm_sqrt(b0[0]*b0[0]+b0[1]*b0[1]+b0[2]*b0[2]);
    T u0[3]={T(1),T(0),T(0)};
    if(n0>tiny){T r=T(1)/n0;u0[0]=b0[0]*r;u0[1]=b0[1]*r;u0[2]=b0[2]*r;}
    T p=u0[0]*b1[0]+u0[1]*b1[1]+u0[2]*b1[2];
    T u1[3]={b1[0]-p*u0[0],b1[1]-p*u0[1],b1[2]-p*u0[2]};
    T n1=mpm_sqrt(u1[0]*u1[0]+u1[1]*u1[1]+u1[2]*u1[2]);
    if(n1>tiny*T(100)*(n0>T(1)?n0:T(1))){T r=T(1)/n1;u1[0]*=r;u1[1]*=r;u1[2]*=r;}
    else{ // any unit vector orthogonal to u0
        int m=0;if(mpm_abs(u0[1])<mpm_abs(u0[m])) m=1;if(mpm_abs(u0[2])<mpm_abs(u0[m])) m=2;
        T e[3]={T(0),T(0),T(0)};e[m]=T(1);T q=u0[m];
        u1[0]=e[0]-q*u0[0];u1[1]=e[1]-q*u0[1];u1[2]=e[2]-q*u0[2];
        T r=T(1)/mpm_sqrt(u1[0]*u1[0]+u1[1]*u1[1]+u1[2]*u1[2]);u1[0]*=r;u1[1]*=r;u1[2]*=r;}
    T u2[3]={u0[1]*u1[2]-u0[2]*u1[1],u0[2]*u1[0]-u0[0]*u1[2],u0[0]*u1[1]-u0[1]*u1[0]};
#pragma unroll
    for(int k=0;k<3;++k){U[3*k]=u0[k];U[3*k+1]=u1[k];U[3*k+2]=u2[k];}
    s[0]=u0[0]*b0[0]+u0[1]*b0[1]+u0[2]*b0[2];
    s[1]=u1[0]*b1[0]+u1[1]*b1[1]+u1[2]*b1[2];
    s[2]=u2[0]*b2[0]+u2[1]*b2[1]+u2[2]*b2[2];
#pragma unroll
    for(int k=0;k<9;++k) V[k]=v[k];
}

// ---- constitutive model (reference MPM_Constitutive_Model.cpp:32-76) ----
struct Plasticity { int plastic; double hardening,compression_yield,stretching_yield,hardening_max; };

// 1/sqrt(x) for x within 1e-4 of 1: 1 - e/2 + 3e^2/8 - 5e^3/16 with e = x - 1 (next term
// 35e^4/128, below 3e-17); otherwise the root and the division.
template<class T> MPM_HD T rsqrt_near1(T x)
{
    const T e=x-T(1);
    if(mpm_abs(e)<=T(1e-4)) return T(1)-e*(T(0.5)-e*(T(0.375)-T(0.3125)*e));
    return T(1)/mpm_sqrt(x);
}
// Columns of V made orthonormal in T (Gram-Schmidt, then a cross product for the third).
// Columns that are already unit length to ~1e-7 (an FP32 solution) take the series for
// the inverse norms.
template<class T> MPM_HD void orthonormalize3(T* v)
{
    T n=rsqrt_near1(v[0]*v[0]+v[3]*v[3]+v[6]*v[6]);
    v[0]*=n;v[3]*=n;v[6]*=n;
    const T p=v[0]*v[1]+v[3]*v[4]+v[6]*v[7];
    v[1]-=p*v[0];v[4]-=p*v[3];v[7]-=p*v[6];
    n=rsqrt_near1(v[1]*v[1]+v[4]*v[4]+v[7]*v[7]);
    v[1]*=n;v[4]*=n;v[7]*=n;
    v[2]=v[3]*v[7]-v[6]*v[4];v[5]=v[6]*v[1]-v[0]*v[7];v[8]=v[0]*v[4]-v[3]*v[1];
}

// Refines an approximate polar rotation R of F (R close to the exact factor R*, F = R* S*
// with S* symmetric): the skew correction W with W S + S W = S - S^T (S = R^T F) is the
// first-order rotation error (the same 3x3 system as dR, reference
// MPM_Constitutive_Model.h:56-69); R <- R (I + W), then (if `bjorck`) one Bjorck step
// R <- R (3I - R^T R)/2 restores orthonormality. Each pass squares the error, so from an
// FP32 start one pass without the Bjorck step leaves an O(1e-14) error, far below the FP32
// rounding of the stored result.
template<class T> MPM_HD T recip(T x);
template<> MPM_HD float recip<float>(float x){return 1.f/x;}
template<> MPM_HD double recip<double>(double x)
{   // FP32 seed and two Newton steps: each step squares the relative error (1e-7 -> 1e-14
    // -> below FP64 rounding), so the result is 1/x to FP64 rounding error. The FP32 seed
    // needs |x| inside the FP32 normal range; outside it (never for the O(1) determinants
    // the polar refinement passes) the plain FP64 division is used.
    const double ax=x<0.?-x:x;
    if(!(ax>=1e-37&&ax<=1e37)) return 1.0/x;
#ifdef __CUDA_ARCH__
    double y=(double)__frcp_rn((float)x);
#else
    double y=(double)(1.f/(float)x);
#endif
    y=y*(2.0-x*y);y=y*(2.0-x*y);
    return y;
}
template<class T> MPM_HD void polar_refine3(const T* F,T* R,bool bjorck=true)
{
    T S[9];mat_mul_at(R,F,S);
    const T s01=T(0.5)*(S[1]+S[3]),s02=T(0.5)*(S[2]+S[6]),s12=T(0.5)*(S[5]+S[7]);
    const T k00=S[4]+S[0],k01=s12,k02=-s02,k11=S[8]+S[0],k12=s01,k22=S[8]+S[4];
    const T L0=S[3]-S[1],L1=S[6]-S[2],L2=S[7]-S[5];
    const T c00=k11*k22-k12*k12,c01=k02*k12-k01*k22,c02=k01*k12-k02*k11;
    const T c11=k00*k22-k02*k02,c12=k01*k02-k00*k12,c22=k00*k11-k01*k01;
    const T inv=recip<T>(k00*c00+k01*c01+k02*c02);
    const T a=(c00*L0+c01*L1+c02*L2)*inv,b=(c01*L0+c11*L1+c12*L2)*inv,c=(c02*L0+c12*L1+c22*L2)*inv;
    T Rn[9];
#pragma unroll
    for(int i=0;i<3;++i){
        const T r0=R[3*i],r1=R[3*i+1],r2=R[3*i+2];
        Rn[3*i]=r0+r1*a+r2*b;Rn[3*i+1]=r1-r0*a+r2*c;Rn[3*i+2]=r2-r0*b-r1*c;}
    if(!bjorck){
#pragma unroll
        for(int k=0;k<9;++k) R[k]=Rn[k];
        return;}
    T G[9];mat_mul_at(Rn,Rn,G);
#pragma unroll
    for(int k=0;k<9;++k) G[k]=(k%4==0?T(1.5):T(0))-T(0.5)*G[k];
    mat_mul(Rn,G,R);
}

// Sum of the six products sum_k (a_k b_k - c_k d_k) over k = 0..2, evaluated as if in twice
// FP32 precision and then rounded: Dot2 (Ogita, Rump & Oishi, "Accurate sum and dot
// product", SIAM J. Sci. Comput. 26, 2005). Each product is split exactly into p + e with
// one fused multiply-add (e = fma(a, b, -p)), the p's are summed with Knuth's error-free
// TwoSum and all error terms are added at the end. The error is below
// 2^-24 |result| + (6 * 2^-24)^2 sum |terms|.
MPM_HD float dot2_skew3(const float* a,const float* b,const float* c,const float* d,int sa,int sb)
{
    float s=0.f,err=0.f;
#pragma unroll
    for(int k=0;k<6;++k){
        const int i=k>>1;
        const float x=(k&1)?-c[sa*i]:a[sa*i],y=(k&1)?d[sb*i]:b[sb*i];
        const float p=x*y,e=fmaf(x,y,-p);              // x y = p + e exactly
        const float t=s+p,z=t-s,q=(s-(t-z))+(p-z);     // s + p = t + q exactly (TwoSum)
        s=t;err+=q+e;}
    return s+err;
}

// det F of an FP32 matrix as the FP64 determinant would round it: the six triple products
// a_i a_j a_k each split into an exact product pair of a_i a_j (one FMA) times a_k (again
// split exactly; the pair's low part times a_k adds an error below 2^-48), summed with
// TwoSum and the error terms added at the end (Dot2). Used by the mixed variant, where the
// FP64 pipe runs at 1/64 of the FP32 rate.
MPM_HD float det3_dot2(const float* a)
{
    const int idx[6][3]={{0,4,8},{1,5,6},{2,3,7},{2,4,6},{0,5,7},{1,3,8}};
    float s=0.f,err=0.f;
#pragma unroll
    for(int t=0;t<6;++t){
        const float x=a[idx[t][0]],y=a[idx[t][1]],z=a[idx[t][2]];
        const float p=x*y,e=fmaf(x,y,-p);               // x y = p + e exactly
        float q=p*z;const float eq=fmaf(p,z,-q);        // p z = q + eq exactly
        float r=fmaf(e,z,eq);                            // the small parts of x y z
        if(t>=3){q=-q;r=-r;}
        const float u=s+q,zz=u-s,c=(s-(u-zz))+(q-zz);    // TwoSum
        s=u;err+=c+r;}
    return s+err;
}

// Mixed-precision form of one polar_refine3 pass without the Bjorck step, for FP32 F and an
// FP32 rotation R. The correction W is ~1e-7, so only its source needs more than FP32: the
// skew part L of R^T F, a difference of nearly equal sums. L is evaluated to twice FP32
// precision by dot2_skew3 (products split exactly, sums compensated), which gives the
// same rounded L as an FP64 evaluation (where the FP32 products are exact) without any
// FP64 operation: on GB300 the FP64 rate is 1/64 of FP32, and the FP64 form cost about a
// fifth of the whole P2G on the 64-scene batch. The symmetric 3x3 system for W and the
// update R + R W stay in FP32: their relative errors (~1e-7) scale W, i.e. ~1e-14
// absolute, far below the FP32 rounding of the stored rotation.
MPM_HD void polar_refine_mixed(const float* F,float* R)
{
    float S[9];mat_mul_at(R,F,S);
    const float s01=0.5f*(S[1]+S[3]),s02=0.5f*(S[2]+S[6]),s12=0.5f*(S[5]+S[7]);
    const float k00=S[4]+S[0],k01=s12,k02=-s02,k11=S[8]+S[0],k12=s01,k22=S[8]+S[4];
    // L0 = sum_k R[k][1] F[k][0] - R[k][0] F[k][1], L1 = (2,0)-(0,2), L2 = (2,1)-(1,2)
    const float l0=dot2_skew3(R+1,F,R,F+1,3,3),l1=dot2_skew3(R+2,F,R,F+2,3,3),l2=dot2_skew3(R+2,F+1,R+1,F+2,3,3);
    const float c00=k11*k22-k12*k12,c01=k02*k12-k01*k22,c02=k01*k12-k02*k11;
    const float c11=k00*k22-k02*k02,c12=k01*k02-k00*k12,c22=k00*k11-k01*k01;
    const float inv=1.f/(k00*c00+k01*c01+k02*c02);
    const float a=(c00*l0+c01*l1+c02*l2)*inv,b=(c01*l0+c11*l1+c12*l2)*inv,c=(c02*l0+c12*l1+c22*l2)*inv;
    float Rn[9];
#pragma unroll
    for(int i=0;i<3;++i){
        const float r0=R[3*i],r1=R[3*i+1],r2=R[3*i+2];
        Rn[3*i]=r0+(r1*a+r2*b);Rn[3*i+1]=r1+(r2*c-r0*a);Rn[3*i+2]=r2-(r0*b+r1*c);}
#pragma unroll
    for(int k=0;k<9;++k) R[k]=Rn[k];
}

// Precompute: SVD of Fe, clamp of the singular values to [cy, sy], Jp update (det of the
// reference's Fp <- V S^-1 U^T Fe Fp), Fe <- U S_hat V^T, hardened Lame parameters,
// Re = U V^T. Writes Fe, Jp in place (rounded to T).
//
// TS == float: everything in FP32. TS == double (mixed and FP64 variants): the SVD is
// first done in FP32. If those singular values lie inside [cy, sy] by a margin far above
// the FP32 error, no clamp happens in exact arithmetic, so Fe and Jp are unchanged and
// only the polar rotation Re is needed, refined in FP64 from the FP32 U V^T by
// polar_refine3. Otherwise the FP64 Jacobi SVD runs, warm-started from the FP32 V, and the
// clamp and reconstruction are done in FP64.
template<class T,class TS> MPM_HD void precompute(T* Fe,T& Jp,const T lambda0,const T mu0,
    const int plastic,const T hardening,const T cy,const T sy,const T hardening_max,
    T* Re,T& lambda,T& mu,T& Je)
{
    float F32[9],U32[9],s32[3],V32[9];
#pragma unroll
    for(int k=0;k<9;++k) F32[k]=(float)Fe[k];
    svd3<float>(F32,U32,s32,V32);
    const bool fp32_only=sizeof(TS)==4;
    const float margin=1e-5f;
    const bool inside=s32[0]<(float)sy-margin&&s32[2]>(float)cy+margin;
    if(fp32_only||(plastic&&!inside)){
        TS F[9],U[9],s[3],V[9];
#pragma unroll
        for(int k=0;k<9;++k) F[k]=(TS)Fe[k];
        if(fp32_only){
#pragma unroll
            for(int k=0;k<9;++k){U[k]=(TS)U32[k];V[k]=(TS)V32[k];}
#pragma unroll
            for(int k=0;k<3;++k) s[k]=(TS)s32[k];}
        else{
            TS V0[9];
#pragma unroll
            for(int k=0;k<9;++k) V0[k]=(TS)V32[k];
            orthonormalize3(V0);
            // the mixed variant stores Fe, Jp and Re in FP32: an FP64 SVD to 1e-12 relative
            // (one sweep from the FP32 start, as a rule) is four orders below that rounding
            svd3<TS,4>(F,U,s,V,V0,sizeof(T)==4?TS(1e-12):TS(0));}
        const TS prod_s=s[0]*s[1]*s[2];
        if(plastic){
            const TS tsy=(TS)sy,tcy=(TS)cy;
#pragma unroll
            for(int i=0;i<3;++i){if(s[i]>tsy) s[i]=tsy;if(s[i]<tcy) s[i]=tcy;}
            const TS prod_hat=s[0]*s[1]*s[2];
            Jp=(T)((TS)Jp*(prod_s/prod_hat));
#pragma unroll
            for(int i=0;i<3;++i)
#pragma unroll
                for(int j=0;j<3;++j) Fe[3*i+j]=(T)(U[3*i]*s[0]*V[3*j]+U[3*i+1]*s[1]*V[3*j+1]+U[3*i+2]*s[2]*V[3*j+2]);}
        Je=(T)(s[0]*s[1]*s[2]);
        TS R[9];mat_mul_bt(U,V,R);
#pragma unroll
        for(int k=0;k<9;++k) Re[k]=(T)R[k];}
    else{
        float R32[9];mat_mul_bt(U32,V32,R32);
        if constexpr(sizeof(T)==8){
            // FP64 variant: to FP64 accuracy
            TS F[9],R[9];
#pragma unroll
            for(int k=0;k<9;++k){F[k]=(TS)Fe[k];R[k]=(TS)R32[k];}
            polar_refine3(F,R);polar_refine3(F,R);
#pragma unroll
            for(int k=0;k<9;++k) Re[k]=(T)R[k];
            Je=(T)det3(F);}
        else{
            // mixed (FP32 Fe and Re): the rounding-sensitive skew residual and det Fe to
            // twice FP32 precision (what FP64 evaluation rounds to), without FP64 operations
            polar_refine_mixed(F32,R32);
#pragma unroll
            for(int k=0;k<9;++k) Re[k]=(T)R32[k];
            Je=(T)det3_dot2(F32);}}
    if(plastic){
        T power=hardening*(T(1)-Jp);if(power>hardening_max) power=hardening_max;
        const T e=mpm_exp<T>(power);
        lambda=e*lambda0;mu=e*mu0;}
    else{lambda=lambda0;mu=mu0;}
}

// First Piola-Kirchhoff stress P = 2 mu (Fe - Re) + lambda (Je-1) cof(Fe), reference :63-67.
template<class T> MPM_HD void stress_P(const T* Fe,const T* Re,const T lambda,const T mu,const T Je,T* P)
{
    T H[9];cofactor3(Fe,H);
    const T c=lambda*(Je-T(1)),m2=T(2)*mu;
#pragma unroll
    for(int k=0;k<9;++k) P[k]=m2*(Fe[k]-Re[k])+c*H[k];
}

// Differential of P along dF, reference :71-76 with dR from MPM_Constitutive_Model.h:56-69:
// dP = 2 mu (dF - dR) + lambda (H:dF) H + lambda (Je-1) dH, with R^T dR the skew matrix W
// solving W S + S W = M - M^T (M = R^T dF, S = R^T Fe), a 3x3 system solved by the adjugate.
// Je and H are recomputed from Fe (Je = det Fe, H = cof Fe).
template<class T> MPM_HD void dP_dF(const T* Fe,const T* Re,const T lambda,const T mu,const T* dF,T* dP)
{
    T H[9];cofactor3(Fe,H);
    const T Je=det3(Fe);
    T M[9],S[9];mat_mul_at(Re,dF,M);mat_mul_at(Re,Fe,S);
    const T k00=S[4]+S[0],k01=S[7],k02=-S[6];
    const T k11=S[8]+S[0],k12=S[3];
    const T k22=S[8]+S[4];
    const T L0=M[3]-M[1],L1=M[6]-M[2],L2=M[7]-M[5];
    // symmetric K: adjugate
    const T c00=k11*k22-k12*k12,c01=k02*k12-k01*k22,c02=k01*k12-k02*k11;
    const T c11=k00*k22-k02*k02,c12=k01*k02-k00*k12,c22=k00*k11-k01*k01;
    const T det=k00*c00+k01*c01+k02*c02;
    const T inv=T(1)/det;
    const T a=(c00*L0+c01*L1+c02*L2)*inv;
    const T b=(c01*L0+c11*L1+c12*L2)*inv;
    const T c=(c02*L0+c12*L1+c22*L2)*inv;
    // dR = R W, W = [[0,-a,-b],[a,0,-c],[b,c,0]]
    T dR[9];
#pragma unroll
    for(int i=0;i<3;++i){
        const T r0=Re[3*i],r1=Re[3*i+1],r2=Re[3*i+2];
        dR[3*i]  = r1*a+r2*b;
        dR[3*i+1]=-r0*a+r2*c;
        dR[3*i+2]=-r0*b-r1*c;}
    T dH[9];cofactor3_diff(Fe,dF,dH);
    T HdF=T(0);
#pragma unroll
    for(int k=0;k<9;++k) HdF+=H[k]*dF[k];
    const T m2=T(2)*mu,lh=lambda*HdF,lj=lambda*(Je-T(1));
#pragma unroll
    for(int k=0;k<9;++k) dP[k]=m2*(dF[k]-dR[k])+lh*H[k]+lj*dH[k];
}

} // namespace mpm
