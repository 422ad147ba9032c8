// Host-side checks of the per-particle 3x3 routines of the sm_103a kernels
// (non_ficks_diffusion_gb300/csrc/mpm_math.cuh), built with nvcc as host code and run on
// the CPU by tests/test_math_host.py. Prints one line of "name value" pairs.
//   polar_mixed_ulp  max |R_mixed - R_fp64| / 2^-23: the mixed polar refinement against one
//                    FP64 pass from the same FP32 rotation, rounded to FP32
//   polar_orth       max |R^T R - I| of the mixed result
//   svd_recon        max |U diag(s) V^T - F| / |F| of the FP64 SVD warm-started from FP32
//   svd_orth         max |U^T U - I|, |V^T V - I| of that SVD
//   rot_small        max relative difference of the near-diagonal Jacobi rotation (series)
//                    from the closed form, over |r| <= 1e-4
#include "mpm_math.cuh"
#include <cmath>
#include <cstdio>
#include <random>

using namespace mpm;

static void rotation(std::mt19937_64& g,double* R)
{
    std::normal_distribution<double> n(0.,1.);
    double q[4];double s=0;for(double& x:q){x=n(g);s+=x*x;}
    s=1./std::sqrt(s);for(double& x:q) x*=s;
    const double w=q[0],x=q[1],y=q[2],z=q[3];
    const double M[9]={1-2*(y*y+z*z),2*(x*y-w*z),2*(x*z+w*y),
                       2*(x*y+w*z),1-2*(x*x+z*z),2*(y*z-w*x),
                       2*(x*z-w*y),2*(y*z+w*x),1-2*(x*x+y*y)};
    for(int k=0;k<9;++k) R[k]=M[k];
}

int main()
{
    std::mt19937_64 g(20261203);
    std::uniform_real_distribution<double> u(-1.,1.);
    double polar_ulp=0,polar_orth=0,recon=0,orth=0;
    for(int it=0;it<20000;++it){
        // F = R0 S0, S0 symmetric positive definite: stretches of +-20 % (inside and
        // outside a snow yield band) and a few near-degenerate ones
        double R0[9],Q[9];rotation(g,R0);rotation(g,Q);
        const double spread=(it%4==0)?1e-6:0.2;
        double sv[3];for(double& x:sv) x=1.+spread*u(g);
        double S0[9];
        for(int i=0;i<3;++i) for(int j=0;j<3;++j){
            double a=0;for(int k=0;k<3;++k) a+=Q[3*i+k]*sv[k]*Q[3*j+k];S0[3*i+j]=a;}
        double Fd[9];mat_mul(R0,S0,Fd);
        float F[9];for(int k=0;k<9;++k) F[k]=(float)Fd[k];
        // the FP32 SVD and its rotation, as in the plasticity update
        float U32[9],s32[3],V32[9],R32[9];
        svd3<float>(F,U32,s32,V32);
        mat_mul_bt(U32,V32,R32);
        // mixed refinement
        float Rm[9];for(int k=0;k<9;++k) Rm[k]=R32[k];
        polar_refine_mixed(F,Rm);
        // one FP64 pass from the same start
        double Fdd[9],Rd[9];for(int k=0;k<9;++k){Fdd[k]=F[k];Rd[k]=R32[k];}
        polar_refine3(Fdd,Rd,false);
        for(int k=0;k<9;++k){
            const double d=std::fabs((double)Rm[k]-(double)(float)Rd[k])/std::ldexp(1.,-23);
            if(d>polar_ulp) polar_ulp=d;}
        double Rmd[9],G[9];for(int k=0;k<9;++k) Rmd[k]=Rm[k];
        mat_mul_at(Rmd,Rmd,G);
        for(int k=0;k<9;++k){const double d=std::fabs(G[k]-(k%4==0?1.:0.));if(d>polar_orth) polar_orth=d;}
        // FP64 SVD warm-started from the FP32 V, to FP64 epsilon
        double V0[9];for(int k=0;k<9;++k) V0[k]=V32[k];
        orthonormalize3(V0);
        double U[9],s[3],V[9];
        svd3<double,4>(Fdd,U,s,V,V0,0.);
        double fn=0;for(int k=0;k<9;++k) fn=std::fmax(fn,std::fabs(Fdd[k]));
        for(int i=0;i<3;++i) for(int j=0;j<3;++j){
            double a=0;for(int k=0;k<3;++k) a+=U[3*i+k]*s[k]*V[3*j+k];
            const double d=std::fabs(a-Fdd[3*i+j])/fn;if(d>recon) recon=d;}
        double GU[9],GV[9];mat_mul_at(U,U,GU);mat_mul_at(V,V,GV);
        for(int k=0;k<9;++k){
            const double e=(k%4==0?1.:0.);
            orth=std::fmax(orth,std::fmax(std::fabs(GU[k]-e),std::fabs(GV[k]-e)));}
    }
    // the rotation series against the closed form
    double rot=0;
    for(int it=0;it<100000;++it){
        const double r=1e-4*u(g);
        if(r==0.) continue;
        const double theta=1./(2.*r);
        const double t_exact=(theta>=0?1.:-1.)/(std::fabs(theta)+std::sqrt(theta*theta+1.));
        const double c_exact=1./std::sqrt(t_exact*t_exact+1.);
        const double r2=r*r,t=r*(1.-r2+2.*r2*r2),t2=t*t,c=1.-t2*(0.5-0.375*t2);
        rot=std::fmax(rot,std::fmax(std::fabs(t-t_exact)/std::fabs(t_exact),std::fabs(c-c_exact)));
    }
    std::printf("polar_mixed_ulp %.3g polar_orth %.3g svd_recon %.3g svd_orth %.3g rot_small %.3g\n",
                polar_ulp,polar_orth,recon,orth,rot);
    return 0;
}
