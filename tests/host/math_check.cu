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
//   upd_ulp / upd_frac_gt1
//                    the mixed plasticity update (FP32 state, FP64 SVD/polar) against the
//                    FP64 one on the same FP32 inputs, rounded to FP32: the largest
//                    difference of Fe, Jp, Re, Je in units of the FP32 spacing (at the
//                    matrix scale for Fe and Re), and the fraction more than one apart
//   upd_clamped      fraction of the cases that clamped a singular value
//   det_mismatch / det_ulp
//                    det3_dot2 (the mixed variant's det Fe) against the FP64 determinant of
//                    the same FP32 matrix rounded to FP32, over 200,000 matrices: how many
//                    differ, and by how many FP32 spacings at most
//   svd32_recon / svd32_orth
//                    the FP32 SVD (cold start, as the FP32 path and the first stage of the
//                    others run it): max |U diag(s) V^T - F| / |F| and max |U^T U - I|,
//                    |V^T V - I|, evaluated in FP64
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

// |a - round(ref)| in units of the FP32 spacing at max(|ref|, scale): entries of O(1)
// matrices are measured against the spacing at the matrix scale, not at their own (small)
// value
static double ulps(float a,double ref,double scale)
{
    const float r=(float)ref;
    const float m=(float)std::fmax(std::fabs(ref),scale);
    const double sp=(double)std::nextafter(m,INFINITY)-(double)m;
    return std::fabs((double)a-(double)r)/sp;
}

int main()
{
    std::mt19937_64 g(20261203);
    std::uniform_real_distribution<double> u(-1.,1.);
    double polar_ulp=0,polar_orth=0,recon=0,orth=0,upd_ulp=0,recon32=0,orth32=0;
    long upd_gt1=0,upd_n=0,upd_clamped=0;
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
        {
            double fn32=0;for(int k=0;k<9;++k) fn32=std::fmax(fn32,std::fabs((double)F[k]));
            for(int i=0;i<3;++i) for(int j=0;j<3;++j){
                double a=0;for(int k=0;k<3;++k) a+=(double)U32[3*i+k]*s32[k]*(double)V32[3*j+k];
                recon32=std::fmax(recon32,std::fabs(a-(double)F[3*i+j])/fn32);}
            for(int i=0;i<3;++i) for(int j=0;j<3;++j){
                double gu=0,gv=0;
                for(int k=0;k<3;++k){gu+=(double)U32[3*k+i]*U32[3*k+j];gv+=(double)V32[3*k+i]*V32[3*k+j];}
                const double e=(i==j?1.:0.);
                orth32=std::fmax(orth32,std::fmax(std::fabs(gu-e),std::fabs(gv-e)));}
        }
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
        // the whole plasticity update, snow band [1 - 2.5e-2, 1 + 7.5e-3]
        {
            float Fm[9],Rm2[9],lam_m,mu_m,Je_m,Jp_m=1.f+0.1f*(float)u(g);
            double Fx[9],Rx[9],lam_x,mu_x,Je_x,Jp_x=Jp_m;
            for(int k=0;k<9;++k){Fm[k]=F[k];Fx[k]=F[k];}
            precompute<float,double>(Fm,Jp_m,1e4f,2e4f,1,10.f,0.975f,1.0075f,10.f,Rm2,lam_m,mu_m,Je_m);
            precompute<double,double>(Fx,Jp_x,1e4,2e4,1,10.,0.975,1.0075,10.,Rx,lam_x,mu_x,Je_x);
            bool cl=false;
            for(int k=0;k<9;++k) if(Fm[k]!=F[k]) cl=true;
            upd_clamped+=cl;
            double d[20];int nd=0;
            double fs=0;for(int k=0;k<9;++k) fs=std::fmax(fs,std::fabs(Fx[k]));
            for(int k=0;k<9;++k){d[nd++]=ulps(Fm[k],Fx[k],fs);d[nd++]=ulps(Rm2[k],Rx[k],1.);}
            d[nd++]=ulps(Jp_m,Jp_x,0.);d[nd++]=ulps(Je_m,Je_x,0.);
            for(int k=0;k<nd;++k){upd_ulp=std::fmax(upd_ulp,d[k]);upd_gt1+=d[k]>1.;upd_n++;}
        }
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
    // det3_dot2 against the FP64 determinant of the same FP32 matrix, rounded to FP32:
    // matrices near the yield band (a rotation times singular values within 3 % of 1) and
    // general ones (entries in [-2, 2])
    long long det_mismatch=0;double det_ulp=0;
    for(int it=0;it<200000;++it){
        float F32[9];
        if(it&1){double R[9],S[9];rotation(g,R);rotation(g,S);
            const double sv[3]={1.+0.03*u(g),1.+0.03*u(g),1.+0.03*u(g)};
            for(int i=0;i<3;++i) for(int j=0;j<3;++j){double a=0;for(int k=0;k<3;++k) a+=R[3*i+k]*sv[k]*S[3*j+k];F32[3*i+j]=(float)a;}}
        else for(int k=0;k<9;++k) F32[k]=(float)(2.*u(g));
        double Fd[9];for(int k=0;k<9;++k) Fd[k]=F32[k];
        const float ref=(float)det3(Fd),got=det3_dot2(F32);
        if(got!=ref){det_mismatch++;det_ulp=std::fmax(det_ulp,std::fabs((double)got-(double)ref)/std::fmax(std::ldexp(1.,-149),
            std::fabs(std::nextafter(ref,2.f*ref+1.f)-ref)));}
    }
    std::printf("polar_mixed_ulp %.3g polar_orth %.3g svd_recon %.3g svd_orth %.3g rot_small %.3g "
                "upd_ulp %.3g upd_frac_gt1 %.3g upd_clamped %.3g svd32_recon %.3g svd32_orth %.3g det_mismatch %lld det_ulp %.3g\n",
                polar_ulp,polar_orth,recon,orth,rot,upd_ulp,(double)upd_gt1/(double)upd_n,(double)upd_clamped/20000.,
                recon32,orth32,det_mismatch,det_ulp);
    return 0;
}
