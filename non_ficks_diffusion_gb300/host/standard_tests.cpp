// standard_tests.cpp — scene presets (include/mpm_scenes.h) and the reference's default
// scene constants (mpm_default_scene). Host-only C++: it is linked into the GPU library and,
// for the CPU baseline, into the oracle's library, so that process loads no GPU code.
#include "mpm_scenes.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace {

// SplitMix64 (Steele, Lea & Flood, "Fast splittable pseudorandom number generators", 2014)
// as a counter-based hash: every sample is a pure function of its coordinates.
inline uint64_t mix(uint64_t z)
{
    z+=0x9e3779b97f4a7c15ULL;
    z=(z^(z>>30))*0xbf58476d1ce4e5b9ULL;
    z=(z^(z>>27))*0x94d049bb133111ebULL;
    return z^(z>>31);
}
inline uint64_t hash4(uint64_t a,uint64_t b,uint64_t c,uint64_t d){return mix(mix(mix(mix(a)^b)^c)^d);}
inline double unit(uint64_t h){return (double)(h>>11)*(1.0/9007199254740992.0);}   // [0,1)

struct Shape {
    int kind;            // 0 sphere, 1 box
    double c[3],h[3];    // centre; radius in h[0] for spheres, half extents for boxes
    double v[3];
    double E,nu;
    bool inside(const double* x,int d) const
    {
        if(kind==0){double r2=0;for(int a=0;a<d;++a) r2+=(x[a]-c[a])*(x[a]-c[a]);return r2<h[0]*h[0];}
        for(int a=0;a<d;++a) if(std::fabs(x[a]-c[a])>=h[a]) return false;
        return true;
    }
    double lo(int a) const {return c[a]-(kind==0?h[0]:h[a]);}
    double hi(int a) const {return c[a]+(kind==0?h[0]:h[a]);}
};

struct Preset {
    int dim=3;
    int n=128;                 // cells per axis
    int ppc_axis=2;            // samples per cell per axis
    double density=400.;
    double dt=1e-4;
    std::vector<Shape> shapes;
    mpm_scene_desc desc;
    bool random_in_shape=false;// reference-style: N uniform samples per shape instead of a jittered grid
    int per_shape=0;
};

void baseline_desc(Preset& p)
{
    mpm_default_scene(&p.desc);
    mpm_scene_desc& d=p.desc;
    for(int a=0;a<3;++a) d.counts[a]=a<p.dim?p.n:1;
    d.gravity[0]=0;d.gravity[1]=-9.8;d.gravity[2]=0;
    d.flip=0.9;d.cg_abs_tol=0;d.cg_rel_tol=1e-5;d.cg_max_iters=50;d.cg_min_iters=0;d.project=1;
    d.plastic=1;d.hardening=10.;d.compression_yield=1.-2.5e-2;d.stretching_yield=1.+7.5e-3;
    const double w=2.0/p.n;
    int k=0;
    auto add=[&](double nx,double ny,double nz,double sx,double sy,double sz,double mu,int sticky){
        mpm_barrier& b=d.barriers[k++];b.normal[0]=nx;b.normal[1]=ny;b.normal[2]=nz;
        b.surface[0]=sx;b.surface[1]=sy;b.surface[2]=sz;b.mu=mu;b.sticky=sticky;};
    add(0,1,0,0,w,0,0,1);           // sticky ground at y=2dx
    add(1,0,0,w,0,0,0,0);add(-1,0,0,1-w,0,0,0,0);   // slip walls
    add(0,-1,0,0,1-w,0,0,0);
    if(p.dim==3){add(0,0,1,0,0,w,0,0);add(0,0,-1,0,0,1-w,0,0);}
    d.n_barriers=k;
}

Shape sphere(double x,double y,double z,double r,double vx,double vy,double vz,double E=1.4e5,double nu=0.2)
{Shape s;s.kind=0;s.c[0]=x;s.c[1]=y;s.c[2]=z;s.h[0]=s.h[1]=s.h[2]=r;s.v[0]=vx;s.v[1]=vy;s.v[2]=vz;s.E=E;s.nu=nu;return s;}
Shape box(double x,double y,double z,double hx,double hy,double hz,double vx,double vy,double vz,double E=1.4e5,double nu=0.2)
{Shape s;s.kind=1;s.c[0]=x;s.c[1]=y;s.c[2]=z;s.h[0]=hx;s.h[1]=hy;s.h[2]=hz;s.v[0]=vx;s.v[1]=vy;s.v[2]=vz;s.E=E;s.nu=nu;return s;}

// Scene `idx` of the batch (test 104), drawn from the seed. The particle count is drawn
// log-uniformly in [1e4, 1e6] (mean about 2.2e5, so 64 scenes hold about 14M particles);
// the grid extent is drawn among those of {64,128,256}^3 on which that count fits 1-3
// shapes of radius (or half-size) 0.05-0.2 at 8 particles per cell.
void batch_scene(Preset& p,int idx,uint64_t seed)
{
    uint64_t k=0;
    auto r=[&](){return unit(hash4(seed,0x104,(uint64_t)idx,k++));};
    const double target=1e4*std::pow(100.0,r());
    const double vmin=4.18879020478639*0.05*0.05*0.05,vmax=3*8*0.2*0.2*0.2;
    int feasible[3],nf=0;
    for(int n:{64,128,256}){const double v=target/(8.0*n*(double)n*n);if(v>=vmin&&v<=vmax) feasible[nf++]=n;}
    p.dim=3;p.n=nf?feasible[std::min(nf-1,(int)(r()*nf))]:128;
    baseline_desc(p);
    const double E0=0.8e5+r()*1.2e5,xi=5.+r()*5.;
    p.desc.hardening=xi;
    const double V=target/(8.0*p.n*(double)p.n*p.n);
    int ns=1+std::min(2,(int)(r()*3));
    while(ns<3&&V/ns>8*0.2*0.2*0.2) ns++;                     // each shape must fit its share
    double wsum=0,w[3];for(int s=0;s<ns;++s){w[s]=0.5+r();wsum+=w[s];}
    for(int s=0;s<ns;++s){
        const double vs=V*w[s]/wsum;
        const bool is_box=r()<0.5;
        double rad=is_box?std::cbrt(vs/8.0):std::cbrt(vs/4.18879020478639);
        rad=std::min(0.2,std::max(0.05,rad));
        const double m=rad+4.0/p.n;
        const double cx=m+r()*(1-2*m),cy=std::max(m,0.3)+r()*std::max(0.,1-m-std::max(m,0.3)),cz=m+r()*(1-2*m);
        const double sp=3.*r(),th=6.283185307179586*r(),ph=std::acos(2*r()-1);
        const double vx=sp*std::sin(ph)*std::cos(th),vy=sp*std::cos(ph)-1.,vz=sp*std::sin(ph)*std::sin(th);
        p.shapes.push_back(is_box?box(cx,cy,cz,rad,rad,rad,vx,vy,vz,E0):sphere(cx,cy,cz,rad,vx,vy,vz,E0));}
}

bool make_preset(int test,int idx,uint64_t seed,Preset& p)
{
    switch(test){
    case 100:
        p.dim=2;p.n=64;p.ppc_axis=4;baseline_desc(p);
        p.shapes.push_back(sphere(.5,.7,0,.12,0,-2,0));return idx==0;
    case 101:
        p.dim=3;p.n=128;baseline_desc(p);
        p.shapes.push_back(sphere(.5,.6,.5,.15,0,-3,0));return idx==0;
    case 102:
        p.dim=3;p.n=256;baseline_desc(p);
        p.shapes.push_back(sphere(.3,.5,.5,.12,3,0,0));
        p.shapes.push_back(sphere(.7,.52,.5,.12,-3,0,0,1.4e5*1.5));return idx==0;
    case 103:{
        p.dim=3;p.n=512;baseline_desc(p);
        mpm_barrier& b=p.desc.barriers[p.desc.n_barriers++];
        b.normal[0]=-0.5;b.normal[1]=std::sqrt(3.)/2.;b.normal[2]=0;
        b.surface[0]=.5;b.surface[1]=.2;b.surface[2]=.5;b.mu=0;b.sticky=0;
        p.shapes.push_back(box(.5,.44,.5,.25,.04,.25,0,-4,0));return idx==0;}
    case 104:
        if(idx<0||idx>=64) return false;
        batch_scene(p,idx,seed);return true;
    case 18:{
        p.dim=3;p.n=64;p.density=2.;
        mpm_default_scene(&p.desc);
        for(int a=0;a<3;++a) p.desc.counts[a]=p.n;
        p.desc.n_barriers=1;
        mpm_barrier& g=p.desc.barriers[0];g.normal[0]=0;g.normal[1]=1;g.normal[2]=0;g.surface[0]=0;g.surface[1]=.1;g.surface[2]=0;g.mu=0;g.sticky=0;
        p.desc.hardening=10.;p.desc.compression_yield=.95;p.desc.stretching_yield=1.01;
        p.random_in_shape=true;p.per_shape=20000;p.dt=1e-3;
        p.shapes.push_back(sphere(.8,.5,.5,.1,-2,.1,0,30.,.4));
        p.shapes.push_back(sphere(.2,.5,.5,.1,2,.1,0,30.,.4));
        return idx==0;}
    case 19:{
        // mpm_3d/Standard_Tests/Standard_Tests.h:113-150: a ball of EOS fluid (bulk modulus 1,
        // gamma 7) falling at 1 m/s inside a box of slip walls at 0.1 and 0.9, on the grid,
        // time step and sampler of test 18.
        p.dim=3;p.n=64;p.density=2.;
        mpm_default_scene(&p.desc);
        for(int a=0;a<3;++a) p.desc.counts[a]=p.n;
        int k=0;
        auto wall=[&](double nx,double ny,double nz,double sx,double sy,double sz){
            mpm_barrier& b=p.desc.barriers[k++];b.normal[0]=nx;b.normal[1]=ny;b.normal[2]=nz;
            b.surface[0]=sx;b.surface[1]=sy;b.surface[2]=sz;b.mu=0;b.sticky=0;};
        wall(0,1,0,0,.1,0);wall(1,0,0,.1,0,0);wall(-1,0,0,.9,0,0);wall(0,0,1,0,0,.1);wall(0,0,-1,0,0,.9);
        p.desc.n_barriers=k;
        p.desc.material=MPM_MATERIAL_EOS_FLUID;p.desc.bulk_modulus=1.;p.desc.eos_gamma=7.;p.desc.plastic=0;
        p.random_in_shape=true;p.per_shape=20000;p.dt=1e-3;
        p.shapes.push_back(sphere(.5,.5,.5,.1,0,-1,0,30.,.4));
        return idx==0;}
    }
    return false;
}

// Jittered-grid sampling over the union bounding box of the shapes; a sample belongs to
// the first shape that contains it.
template<class F> long long sample(const Preset& p,int idx,uint64_t seed,F&& emit)
{
    const int d=p.dim,k=p.ppc_axis;
    const double dx=1.0/p.n;
    long long count=0;
    if(p.random_in_shape){
        for(size_t s=0;s<p.shapes.size();++s){
            const Shape& sh=p.shapes[s];
            uint64_t t=0;
            for(int i=0;i<p.per_shape;){
                double x[3]={0,0,0};
                for(int a=0;a<d;++a) x[a]=sh.lo(a)+(sh.hi(a)-sh.lo(a))*unit(hash4(seed,(uint64_t)s,t,(uint64_t)a));
                t++;
                if(!sh.inside(x,d)) continue;
                emit(x,sh,(double)(4.18879020478639*sh.h[0]*sh.h[0]*sh.h[0])/p.per_shape*p.density);++i;++count;}}
        return count;
    }
    int lo[3]={0,0,0},hi[3]={0,0,0};
    for(int a=0;a<d;++a){
        double l=1,h=0;for(auto& s:p.shapes){l=std::min(l,s.lo(a));h=std::max(h,s.hi(a));}
        lo[a]=std::max(0,(int)std::floor(l*p.n)-1);hi[a]=std::min(p.n-1,(int)std::floor(h*p.n)+1);}
    double cellvol=1;for(int a=0;a<d;++a) cellvol*=dx;
    int ppc=1;for(int a=0;a<d;++a) ppc*=k;
    const double m=p.density*cellvol/ppc;
    for(int cz=(d==3?lo[2]:0);cz<=(d==3?hi[2]:0);++cz)
    for(int cy=lo[1];cy<=hi[1];++cy)
    for(int cx=lo[0];cx<=hi[0];++cx){
        const uint64_t cell=((uint64_t)cz*4096+(uint64_t)cy)*4096+(uint64_t)cx;
        for(int sidx=0;sidx<ppc;++sidx){
            int sub[3]={sidx%k,(sidx/k)%k,sidx/(k*k)};
            const int cc[3]={cx,cy,cz};
            double x[3]={0,0,0};
            for(int a=0;a<d;++a) x[a]=(cc[a]+(sub[a]+unit(hash4(seed,(uint64_t)idx,cell,(uint64_t)(sidx*3+a))))/k)*dx;
            for(auto& s:p.shapes) if(s.inside(x,d)){emit(x,s,m);++count;break;}}}
    return count;
}

} // namespace

extern "C" {

void mpm_default_scene(mpm_scene_desc* d)
{
    if(!d) return;
    std::memset(d,0,sizeof(*d));
    d->counts[0]=d->counts[1]=d->counts[2]=32;             // -size default (MPM_Example.cpp:863)
    d->gravity[1]=-2.;                                      // MPM_Example.cpp:81
    d->flip=0.9;                                            // :82
    d->cg_abs_tol=1e-7;d->cg_rel_tol=0.;                    // :78
    d->cg_max_iters=10000;d->cg_min_iters=0;                // :79, :711
    d->project=1;
    d->plastic=1;d->hardening=10.;d->compression_yield=0.95;d->stretching_yield=1.01;   // Standard_Tests.h:82-85
    d->hardening_max=(double)FLT_MAX;                       // MPM_Constitutive_Model.h:20
    d->material=MPM_MATERIAL_SNOW;d->bulk_modulus=1e7;d->eos_gamma=7.;   // MPM_Particle.h:56-58
}

mpm_status mpm_preset_scene(int test,int idx,unsigned long long seed,mpm_scene_desc* desc,mpm_preset_info* info)
{
    Preset p;
    if(!make_preset(test,idx,seed,p)) return MPM_BAD_ARG;
    if(desc) *desc=p.desc;
    if(info){
        std::memset(info,0,sizeof(*info));
        info->dim=p.dim;info->scene_count=test==104?64:1;info->dt=p.dt;info->frame_dt=1.0/24.0;info->density=p.density;
        info->n_particles=sample(p,idx,seed,[](const double*,const Shape&,double){});}
    return MPM_OK;
}

mpm_status mpm_preset_particles(int test,int idx,unsigned long long seed,long long capacity,double* X,double* V,double* mass,
                                double* lambda0,double* mu0)
{
    Preset p;
    if(!make_preset(test,idx,seed,p)) return MPM_BAD_ARG;
    const int d=p.dim;
    long long i=0;
    bool overflow=false;
    sample(p,idx,seed,[&](const double* x,const Shape& s,double m){
        if(i>=capacity){overflow=true;return;}
        for(int a=0;a<d;++a){if(X) X[i*d+a]=x[a];if(V) V[i*d+a]=s.v[a];}
        const double mu=s.E/(2.*(1.+s.nu)),lam=s.E*s.nu/((1.+s.nu)*(1.-2.*s.nu));   // MPM_Constitutive_Model.cpp:23-28
        if(mass) mass[i]=m;if(lambda0) lambda0[i]=lam;if(mu0) mu0[i]=mu;
        ++i;});
    return overflow?MPM_CAPACITY:MPM_OK;
}

}
