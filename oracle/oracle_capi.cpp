// oracle_capi.cpp — extern "C" surface of the CPU oracle (TEST INFRASTRUCTURE ONLY).
// Loaded by the tests and by the bench's CPU-baseline leg through ctypes. Never linked
// into the product library. See mpm_oracle.h for what is restated from where.
#include "mpm_oracle.h"
#include <chrono>
#include <algorithm>
#include <memory>
#include <type_traits>

using namespace oracle;

namespace {
struct Handle {
    int d,precision;
    void* sim;
};
template<class S> S* as(Handle* h){return static_cast<S*>(h->sim);}

using S2f=MPM_Oracle<float,float,float,2>;   using S3f=MPM_Oracle<float,float,float,3>;
using S2m=MPM_Oracle<float,double,double,2>; using S3m=MPM_Oracle<float,double,double,3>;
using S2d=MPM_Oracle<double,double,double,2>;using S3d=MPM_Oracle<double,double,double,3>;

// Dispatch on (d, precision): 0 fp32, 1 mixed (fp32 state, fp64 SVD and reductions), 2 fp64.
template<class F> auto dispatch(Handle* h,F&& f)
{
    if(h->d==2){
        if(h->precision==0) return f(as<S2f>(h));
        if(h->precision==1) return f(as<S2m>(h));
        return f(as<S2d>(h));}
    if(h->precision==0) return f(as<S3f>(h));
    if(h->precision==1) return f(as<S3m>(h));
    return f(as<S3d>(h));
}
}

extern "C" {

void* oracle_create(int d,int precision,const SceneParams* p,int threads)
{
    if((d!=2&&d!=3)||precision<0||precision>2||!p) return nullptr;
    Handle* h=new Handle{d,precision,nullptr};
    if(d==2){
        if(precision==0) h->sim=new S2f(*p,threads); else if(precision==1) h->sim=new S2m(*p,threads); else h->sim=new S2d(*p,threads);}
    else{
        if(precision==0) h->sim=new S3f(*p,threads); else if(precision==1) h->sim=new S3m(*p,threads); else h->sim=new S3d(*p,threads);}
    return h;
}

void oracle_destroy(void* hv)
{
    Handle* h=(Handle*)hv;if(!h) return;
    dispatch(h,[](auto* s){delete s;return 0;});
    delete h;
}

int oracle_sizeof_scene_params(){return (int)sizeof(SceneParams);}

// Particle arrays are particle-major doubles: X,V n*d; Fe n*d*d (row-major) or NULL for
// identity; Jp NULL for 1; V0 NULL for "compute at Initialize".
void oracle_add_particles(void* hv,long long n,const double* X,const double* V,const double* mass,
                          const double* lambda0,const double* mu0,const double* Fe,const double* Jp,const double* V0)
{
    Handle* h=(Handle*)hv;
    dispatch(h,[&](auto* s){
        using Sim=std::decay_t<decltype(*s)>;
        constexpr int d=Sim::dim;
        using S=typename Sim::scalar;
        for(long long i=0;i<n;++i){
            S x[3],v[3],F[9];
            for(int a=0;a<d;++a){x[a]=(S)X[i*d+a];v[a]=(S)V[i*d+a];}
            if(Fe) for(int k=0;k<d*d;++k) F[k]=(S)Fe[i*d*d+k];
            s->Add_Particle(x,v,(S)mass[i],(S)lambda0[i],(S)mu0[i],Fe?F:nullptr,Jp?(S)Jp[i]:(S)1,V0?(S)V0[i]:(S)0);}
        return 0;});
}

void oracle_initialize(void* hv){dispatch((Handle*)hv,[](auto* s){s->Initialize();return 0;});}

// Allocate_Particle for n particles (particle-major doubles as in oracle_add_particles);
// ids[i] receives the index each one took.
void oracle_allocate_particles(void* hv,long long n,const double* X,const double* V,const double* mass,
                               const double* lambda0,const double* mu0,int* ids)
{
    dispatch((Handle*)hv,[&](auto* s){
        using Sim=std::decay_t<decltype(*s)>;
        constexpr int d=Sim::dim;
        using S=typename Sim::scalar;
        for(long long i=0;i<n;++i){
            S x[3],v[3];
            for(int a=0;a<d;++a){x[a]=(S)X[i*d+a];v[a]=(S)V[i*d+a];}
            const int id=s->Allocate_Particle(x,v,(S)mass[i],(S)lambda0[i],(S)mu0[i]);
            if(ids) ids[i]=id;}
        return 0;});
}

// Runs one substep; returns the CG iteration count. stop_after as in MPM_Oracle::Advance_Step.
int oracle_advance_step(void* hv,double dt,int stop_after)
{
    return dispatch((Handle*)hv,[&](auto* s){
        using S=typename std::decay_t<decltype(*s)>::scalar;
        s->Advance_Step((S)dt,stop_after);return s->last.cg_iterations;});
}

// Runs k substeps and returns the wall time in seconds (for the CPU baseline).
double oracle_run_substeps(void* hv,int k,double dt)
{
    return dispatch((Handle*)hv,[&](auto* s){
        using S=typename std::decay_t<decltype(*s)>::scalar;
        auto t0=std::chrono::steady_clock::now();
        for(int i=0;i<k;++i) s->Advance_Step((S)dt,0);
        auto t1=std::chrono::steady_clock::now();
        return std::chrono::duration<double>(t1-t0).count();});
}

long long oracle_num_particles(void* hv){return dispatch((Handle*)hv,[](auto* s){return (long long)s->X.size();});}
long long oracle_num_simulated(void* hv){return dispatch((Handle*)hv,[](auto* s){return (long long)s->simulated.size();});}

void oracle_get_particles(void* hv,double* X,double* V,double* Fe,double* Jp,double* V0,int* valid)
{
    dispatch((Handle*)hv,[&](auto* s){
        constexpr int d=std::decay_t<decltype(*s)>::dim;
        const size_t n=s->X.size();
        for(size_t i=0;i<n;++i){
            for(int a=0;a<d;++a){if(X) X[i*d+a]=s->X[i][a];if(V) V[i*d+a]=s->V[i][a];}
            if(Fe) for(int r=0;r<d;++r) for(int c=0;c<d;++c) Fe[i*d*d+r*d+c]=s->Fe[i].a[r][c];
            if(Jp) Jp[i]=s->Jp[i];if(V0) V0[i]=s->V0[i];if(valid) valid[i]=s->valid[i];}
        return 0;});
}

// Closest cells after the last Update_Particle_Weights (n*d ints).
void oracle_get_cells(void* hv,int* cells)
{
    dispatch((Handle*)hv,[&](auto* s){std::copy(s->cc.begin(),s->cc.end(),cells);return 0;});
}

long long oracle_num_interior(void* hv)
{
    return dispatch((Handle*)hv,[](auto* s){long long n=0;for(size_t l=0;l<s->gsize;++l) if(s->flags[l]&Flag_Interior) n++;return n;});
}

// Interior nodes: coords (n*d ints), m, v (n*d), v* (n*d), f (n*d).
void oracle_get_interior(void* hv,int* coords,double* m,double* v,double* vs,double* f)
{
    dispatch((Handle*)hv,[&](auto* s){
        constexpr int d=std::decay_t<decltype(*s)>::dim;
        long long k=0;
        for(size_t l=0;l<s->gsize;++l){if(!(s->flags[l]&Flag_Interior)) continue;
            int c[d];s->Node_Coords(l,c);
            for(int a=0;a<d;++a){if(coords) coords[k*d+a]=c[a];if(v) v[k*d+a]=s->gv[l][a];if(vs) vs[k*d+a]=s->gvs[l][a];if(f) f[k*d+a]=s->gf[l][a];}
            if(m) m[k]=s->gm[l];k++;}
        return 0;});
}

void oracle_flag_counts(void* hv,long long* out){dispatch((Handle*)hv,[&](auto* s){s->Flag_Counts(out);return 0;});}

void oracle_last_stats(void* hv,StepStats* out){dispatch((Handle*)hv,[&](auto* s){*out=s->last;return 0;});}

double oracle_max_particle_velocity(void* hv){return dispatch((Handle*)hv,[](auto* s){return (double)s->Max_Particle_Velocity();});}

// MPM_Driver::Advance_To_Target_Time (MPM_Driver.cpp:55-80) in the simulation's scalar type,
// as the reference's driver computes it: before every substep dt = clamp(cfl dx /
// max(Max_Particle_Velocity, 1e-2), 1e-6, 5e-3); the substep that would overshoot (within
// 0.1 %) lands on the target and ends the advance, and one that leaves less than two steps
// takes half the rest. *time is the driver's clock (advanced); stops after max_substeps.
// Returns the number of substeps.
int oracle_advance_to_time(void* hv,double* time,double target_time,double cfl,int max_substeps)
{
    return dispatch((Handle*)hv,[&](auto* s){
        using S=typename std::decay_t<decltype(*s)>::scalar;
        const S min_dt=(S)1e-6,max_dt=(S).005,c=(S)cfl,dx_min=s->dx[0],target=(S)target_time;
        S t=(S)*time;
        bool done=false;int k=0;
        for(;!done&&k<max_substeps;++k){
            const S max_v=s->Max_Particle_Velocity();
            S dt=std::max(min_dt,std::min(max_dt,c*dx_min/std::max(max_v,(S)1e-2)));
            if(target-t<dt*(S)1.001){dt=target-t;done=true;}
            else if(target-t<(S)2.*dt) dt=(target-t)*(S).5;
            s->Advance_Step(dt,0);
            t+=dt;}
        *time=(double)t;
        return k;});
}

// ---- math kernels in double, for the finite-difference and known-answer tests ----
static Mat<double,3> M3(const double* a){Mat<double,3> m;for(int i=0;i<3;++i) for(int j=0;j<3;++j) m.a[i][j]=a[i*3+j];return m;}
static void W3(const Mat<double,3>& m,double* a){for(int i=0;i<3;++i) for(int j=0;j<3;++j) a[i*3+j]=m.a[i][j];}
static Mat<double,2> M2(const double* a){Mat<double,2> m;for(int i=0;i<2;++i) for(int j=0;j<2;++j) m.a[i][j]=a[i*2+j];return m;}
static void W2(const Mat<double,2>& m,double* a){for(int i=0;i<2;++i) for(int j=0;j<2;++j) a[i*2+j]=m.a[i][j];}

void oracle_svd(int d,const double* F,double* U,double* s,double* V)
{
    if(d==3){Mat<double,3> u,v;Vec<double,3> sv;SVD(M3(F),u,sv,v);W3(u,U);W3(v,V);for(int i=0;i<3;++i) s[i]=sv[i];}
    else{Mat<double,2> u,v;Vec<double,2> sv;SVD(M2(F),u,sv,v);W2(u,U);W2(v,V);for(int i=0;i<2;++i) s[i]=sv[i];}
}
void oracle_svd_f32(const float* F,float* U,float* s,float* V)
{
    Mat<float,3> f,u,v;Vec<float,3> sv;for(int i=0;i<3;++i) for(int j=0;j<3;++j) f.a[i][j]=F[i*3+j];
    SVD(f,u,sv,v);for(int i=0;i<3;++i){s[i]=sv[i];for(int j=0;j<3;++j){U[i*3+j]=u.a[i][j];V[i*3+j]=v.a[i][j];}}
}

// Unclamped constitutive model at F (Jp=1, not plastic): returns Psi and writes P (d*d).
double oracle_psi_P(int d,const double* F,double lambda,double mu,double* Pout)
{
    PlasticityParams pp{0,0,0,0,0};
    if(d==3){Mat<double,3> f=M3(F);double jp=1;Constitutive<double,3> cm;Precompute<double,double,3>(f,jp,lambda,mu,pp,cm);if(Pout) W3(cm.P(),Pout);return cm.Psi();}
    Mat<double,2> f=M2(F);double jp=1;Constitutive<double,2> cm;Precompute<double,double,2>(f,jp,lambda,mu,pp,cm);if(Pout) W2(cm.P(),Pout);return cm.Psi();
}
// Times_dP_dF at F (not plastic) applied to dF.
void oracle_dP(int d,const double* F,double lambda,double mu,const double* dF,double* out)
{
    PlasticityParams pp{0,0,0,0,0};
    if(d==3){Mat<double,3> f=M3(F);double jp=1;Constitutive<double,3> cm;Precompute<double,double,3>(f,jp,lambda,mu,pp,cm);W3(cm.Times_dP_dF(M3(dF)),out);return;}
    Mat<double,2> f=M2(F);double jp=1;Constitutive<double,2> cm;Precompute<double,double,2>(f,jp,lambda,mu,pp,cm);W2(cm.Times_dP_dF(M2(dF)),out);
}
// Polar rotation of F and its differential along dF.
void oracle_polar_dR(int d,const double* F,const double* dF,double* R,double* dRout)
{
    if(d==3){Mat<double,3> u,v;Vec<double,3> s;Mat<double,3> f=M3(F);SVD(f,u,s,v);Mat<double,3> r=Times_Transpose(u,v);W3(r,R);W3(dR(M3(dF),r,f),dRout);return;}
    Mat<double,2> u,v;Vec<double,2> s;Mat<double,2> f=M2(F);SVD(f,u,s,v);Mat<double,2> r=Times_Transpose(u,v);W2(r,R);W2(dR(M2(dF),r,f),dRout);
}
void oracle_cofactor(int d,const double* F,const double* dF,double* C,double* dC)
{
    if(d==3){W3(Cofactor(M3(F)),C);W3(Times_Cofactor_Matrix_Derivative(M3(F),M3(dF)),dC);return;}
    W2(Cofactor(M2(F)),C);W2(Times_Cofactor_Matrix_Derivative(M2(F),M2(dF)),dC);
}
// Plasticity step on one matrix: returns new Fe, Jp and the hardened (lambda, mu).
void oracle_plasticity(int d,double* F,double* Jp,double lambda0,double mu0,const PlasticityParams* pp,double* lam_mu)
{
    if(d==3){Mat<double,3> f=M3(F);Constitutive<double,3> cm;Precompute<double,double,3>(f,*Jp,lambda0,mu0,*pp,cm);W3(f,F);lam_mu[0]=cm.lambda;lam_mu[1]=cm.mu;return;}
    Mat<double,2> f=M2(F);Constitutive<double,2> cm;Precompute<double,double,2>(f,*Jp,lambda0,mu0,*pp,cm);W2(f,F);lam_mu[0]=cm.lambda;lam_mu[1]=cm.mu;
}
void oracle_weights(double x,double one_over_dx,double* w,double* dw){Compute_Weights(x,one_over_dx,w,dw);}
void oracle_weights_f32(float x,float one_over_dx,float* w,float* dw){Compute_Weights(x,one_over_dx,w,dw);}

}
