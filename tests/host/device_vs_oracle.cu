// Host-side cross-check of the per-particle routines of the sm_103a kernels
// (non_ficks_diffusion_gb300/csrc/mpm_math.cuh, built as host code) against the CPU
// oracle (oracle/mpm_oracle.h) on random deformation gradients; run by
// tests/test_math_host.py. Prints "name value" pairs: maximum relative differences over the
// cases, for FP64 (fp64_*) and for the mixed variant against the oracle's mixed variant
// (mixed_*, in FP32 spacings at the matrix scale).
#include "mpm_math.cuh"
#include "mpm_oracle.h"
#include <cmath>
#include <cstdio>
#include <random>

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
template<class T> static oracle::Mat<T,3> to_mat(const T* a){oracle::Mat<T,3> m;for(int i=0;i<3;++i) for(int j=0;j<3;++j) m.a[i][j]=a[3*i+j];return m;}

int main()
{
    std::mt19937_64 g(7);
    std::uniform_real_distribution<double> u(-1.,1.);
    const oracle::PlasticityParams pp{1,10.,0.975,1.0075,10.};
    double f_upd=0,f_P=0,f_dP=0,f_w=0,m_upd=0;
    for(int it=0;it<20000;++it){
        double A[9],B[9];rotation(g,A);rotation(g,B);
        double sv[3];for(double& x:sv) x=1.+0.2*u(g);
        double F[9];
        for(int i=0;i<3;++i) for(int j=0;j<3;++j){double a=0;for(int k=0;k<3;++k) a+=A[3*i+k]*sv[k]*B[3*j+k];F[3*i+j]=a;}
        const double Jp0=1.+0.1*u(g);
        // FP64 plasticity update
        double Fd[9],Rd[9],lam,mu,Je,Jp=Jp0;for(int k=0;k<9;++k) Fd[k]=F[k];
        mpm::precompute<double,double>(Fd,Jp,1e4,2e4,1,10.,0.975,1.0075,10.,Rd,lam,mu,Je);
        oracle::Mat<double,3> Fo=to_mat(F);double Jpo=Jp0;oracle::Constitutive<double,3> cm;
        oracle::Precompute<double,double,3>(Fo,Jpo,1e4,2e4,pp,cm);
        double fs=0;for(int k=0;k<9;++k) fs=std::fmax(fs,std::fabs(cm.Fe.a[k/3][k%3]));
        for(int k=0;k<9;++k){
            f_upd=std::fmax(f_upd,std::fabs(Fd[k]-cm.Fe.a[k/3][k%3])/fs);
            f_upd=std::fmax(f_upd,std::fabs(Rd[k]-cm.Re.a[k/3][k%3]));}
        f_upd=std::fmax(f_upd,std::fabs(Jp-Jpo)/std::fabs(Jpo));
        f_upd=std::fmax(f_upd,std::fabs(Je-cm.Je)/std::fabs(cm.Je));
        f_upd=std::fmax(f_upd,std::fabs(lam-cm.lambda)/cm.lambda);
        // stress and its differential from the same state
        double Fe[9],Re[9];for(int k=0;k<9;++k){Fe[k]=cm.Fe.a[k/3][k%3];Re[k]=cm.Re.a[k/3][k%3];}
        double P[9];mpm::stress_P(Fe,Re,cm.lambda,cm.mu,cm.Je,P);
        const oracle::Mat<double,3> Po=cm.P();
        double ps=0;for(int k=0;k<9;++k) ps=std::fmax(ps,std::fabs(Po.a[k/3][k%3]));
        for(int k=0;k<9;++k) f_P=std::fmax(f_P,std::fabs(P[k]-Po.a[k/3][k%3])/ps);
        double dF[9];for(double& x:dF) x=1e-3*u(g);
        double dP[9];mpm::dP_dF(Fe,Re,cm.lambda,cm.mu,dF,dP);
        const oracle::Mat<double,3> dPo=cm.Times_dP_dF(to_mat(dF));
        double ds=0;for(int k=0;k<9;++k) ds=std::fmax(ds,std::fabs(dPo.a[k/3][k%3]));
        for(int k=0;k<9;++k) f_dP=std::fmax(f_dP,std::fabs(dP[k]-dPo.a[k/3][k%3])/ds);
        // weights
        const double x=0.5+0.999999*(0.5+0.5*u(g));
        double w[3],dw[3],wo[3],dwo[3];
        mpm::bspline_weights<double>(x,128.,w,dw);oracle::Compute_Weights(x,128.,wo,dwo);
        for(int k=0;k<3;++k) f_w=std::fmax(f_w,std::fmax(std::fabs(w[k]-wo[k]),std::fabs(dw[k]-dwo[k])/128.));
        // mixed: FP32 state, FP64 SVD/polar, against the oracle's mixed form
        float Fm[9],Rm[9],lamm,mum,Jem,Jpm=(float)Jp0;for(int k=0;k<9;++k) Fm[k]=(float)F[k];
        oracle::Mat<float,3> Fmo;for(int k=0;k<9;++k) Fmo.a[k/3][k%3]=Fm[k];
        float Jpmo=Jpm;oracle::Constitutive<float,3> cmm;
        mpm::precompute<float,double>(Fm,Jpm,1e4f,2e4f,1,10.f,0.975f,1.0075f,10.f,Rm,lamm,mum,Jem);
        oracle::Precompute<float,double,3>(Fmo,Jpmo,1e4f,2e4f,pp,cmm);
        const double sp=std::ldexp(1.,-23);
        for(int k=0;k<9;++k){
            m_upd=std::fmax(m_upd,std::fabs((double)Fm[k]-(double)cmm.Fe.a[k/3][k%3])/(sp*std::fmax(1.,fs)));
            m_upd=std::fmax(m_upd,std::fabs((double)Rm[k]-(double)cmm.Re.a[k/3][k%3])/sp);}
        m_upd=std::fmax(m_upd,std::fabs((double)Jpm-(double)Jpmo)/(sp*std::fabs((double)Jpmo)));
    }
    std::printf("fp64_update %.3g fp64_P %.3g fp64_dP %.3g weights %.3g mixed_update_spacings %.3g\n",f_upd,f_P,f_dP,f_w,m_upd);
    return 0;
}
