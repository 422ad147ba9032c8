// mpm_host.h — C++ host surface over the C ABI, mirroring the reference's driver classes
// (MPM_Driver.h:13-36, MPM_Example.h:308-331, mpm_3d/Standard_Tests/Standard_Tests.h) so a
// reference user drives the GB300 substep with the same calls. The per-phase methods that
// the GPU fuses into one substep are kept as no-ops with the reference's names, and
// Update_Particle_Velocities_And_Positions runs the whole substep (mpm_advance_step).
#pragma once
#include "mpm_gb300.h"
#include "mpm_scenes.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <cstdint>
#include <sys/stat.h>
#include <vector>

namespace mpm_host {

inline void check(mpm_status s,const mpm_context* c,const char* what)
{
    if(s==MPM_OK||s==MPM_CG_NOT_CONVERGED) return;
    throw std::runtime_error(std::string(what)+": "+mpm_status_string(s)+(c?std::string(" (")+mpm_last_error(c)+")":std::string()));
}

// MPM_Example<T,3> (MPM_Example.h:227-337) backed by a GPU context.
class MPM_Example
{
  public:
    mpm_config config;
    mpm_context* ctx=nullptr;
    int test_number=101,scene_count=1,last_frame=1,current_frame=0,output_number=0;
    unsigned long long seed=0;
    double cfl=0.1,fixed_dt=0;      // fixed_dt>0 replaces the CFL rule
    double dx_min=1.;               // finest cell size over the scenes (MPM_Driver.cpp:61)
    double frame_rate=24.;
    std::string output_directory="mpm_3d_output";
    bool write_output=false;
    bool restart=false;int restart_frame=0;   // Nova Example's -restart (MPM_Driver.cpp:22-31)
    std::vector<long long> scene_particles;

    MPM_Example(){mpm_default_config(&config);}
    virtual ~MPM_Example(){if(ctx) mpm_destroy(ctx);}

    double Time_At_Frame(int frame) const {return frame/frame_rate;}

    // Standard_Tests::Initialize_Particles (pure virtual in the reference, MPM_Example.h:306)
    virtual void Initialize_Particles(int test_case)
    {
        mpm_preset_info info;mpm_scene_desc desc;
        check(mpm_preset_scene(test_case,0,seed,&desc,&info),nullptr,"preset");
        if(info.dim!=3) throw std::runtime_error("the GPU path is 3D; test "+std::to_string(test_case)+" is 2D");
        scene_count=info.scene_count;
        long long total=0;std::vector<mpm_preset_info> infos(scene_count);std::vector<mpm_scene_desc> descs(scene_count);
        for(int s=0;s<scene_count;++s){check(mpm_preset_scene(test_case,s,seed,&descs[s],&infos[s]),nullptr,"preset");total+=infos[s].n_particles;
            for(int a=0;a<3;++a) dx_min=std::min(dx_min,1.0/descs[s].counts[a]);}
        if(fixed_dt==0) fixed_dt=info.dt;
        config.max_particles=std::max<long long>(config.max_particles,total);
        config.max_scenes=std::max(config.max_scenes,scene_count);
        check(mpm_create(&config,&ctx),nullptr,"mpm_create");
        for(int s=0;s<scene_count;++s){
            int id=0;check(mpm_add_scene(ctx,&descs[s],&id),ctx,"mpm_add_scene");
            const long long n=infos[s].n_particles;
            std::vector<double> X(3*n),V(3*n),m(n),l(n),mu(n);
            check(mpm_preset_particles(test_case,s,seed,n,X.data(),V.data(),m.data(),l.data(),mu.data()),nullptr,"particles");
            mpm_particle_arrays p{};p.n=n;p.dtype=MPM_F64;p.X=X.data();p.V=V.data();p.mass=m.data();p.lambda0=l.data();p.mu0=mu.data();
            check(mpm_add_particles(ctx,id,&p),ctx,"mpm_add_particles");
            scene_particles.push_back(n);}
    }

    // MPM_Example.cpp:152-161
    void Initialize(){Initialize_Particles(test_number);}
    // Phases that the GPU substep fuses; kept for call-for-call compatibility with
    // MPM_Driver::Advance_Step (MPM_Driver.cpp:106-114).
    void Initialize_SPGrid(){}
    void Reset_Grid_Based_Variables(){}
    void Update_Particle_Weights(){}
    void Group_Particles(){}
    void Rasterize_Voxels(){}
    void Rasterize(){}
    void Process_Waiting_Particles(){check(mpm_initialize(ctx),ctx,"mpm_initialize");}
    void Update_Constitutive_Model_State(){}
    void Populate_Simulated_Particles(){}
    // The whole substep: grid build, P2G, plasticity, explicit force, collision, CG, G2P.
    void Update_Particle_Velocities_And_Positions(double dt){check(mpm_advance_step(ctx,dt),ctx,"mpm_advance_step");}
    // MPM_Example.cpp:375-387 (maximum over all scenes)
    double Max_Particle_Velocity() const
    {double m=0;for(int s=0;s<scene_count;++s){double v=0;check(mpm_max_particle_velocity(ctx,s,&v),ctx,"vmax");m=std::max(m,v);}return m;}

    // Write_Output_Files (MPM_Example.cpp:1049-1063) with the particle record of
    // Read_Write_MPM_Particles.h:33-46: a size_t count of valid particles, then X, V (3 floats
    // each), mass and volume (float) per valid particle. One file per scene.
    void Write_Output_Files(int frame) const
    {
        if(!write_output) return;
        ::mkdir(output_directory.c_str(),0755);
        const std::string dir=output_directory+"/"+std::to_string(frame);
        ::mkdir(dir.c_str(),0755);
        for(int s=0;s<scene_count;++s){
            const long long n=scene_particles[s];
            std::vector<float> X(3*n),V(3*n),m(n),v0(n);std::vector<int> valid(n);
            mpm_particle_arrays o{};o.n=n;o.dtype=MPM_F32;o.X=X.data();o.V=V.data();o.mass=m.data();o.V0=v0.data();o.valid=valid.data();
            check(mpm_get_particles(ctx,s,&o),ctx,"mpm_get_particles");
            std::ofstream f(dir+"/particles"+(scene_count>1?"_"+std::to_string(s):std::string()),std::ios::binary);
            size_t count=0;for(int v:valid) count+=v?1:0;
            f.write((const char*)&count,sizeof(count));
            for(long long i=0;i<n;++i){if(!valid[i]) continue;
                f.write((const char*)&X[3*i],12);f.write((const char*)&V[3*i],12);f.write((const char*)&m[i],4);f.write((const char*)&v0[i],4);}}
        Write_Checkpoint(dir);
    }

    // Full-state checkpoint beside the reference's particle file. The reference restarts
    // from X, V, mass and volume only (Read_Write_MPM_Particles.h:21-30), which resets Fe
    // and the plastic state. This record keeps every particle field, the removed flags
    // and the clock, in FP64: "MPMCKPT1", int32 scene count, FP64 time, then per scene an
    // int64 particle count, X, V (3n), Fe (9n), Jp, V0, mass, lambda0, mu0 (n each, FP64)
    // and the int32 valid flags.
    void Write_Checkpoint(const std::string& dir) const
    {
        std::ofstream f(dir+"/checkpoint",std::ios::binary);
        double t=0;check(mpm_get_time(ctx,&t),ctx,"mpm_get_time");
        const int32_t ns=scene_count;
        f.write("MPMCKPT1",8);f.write((const char*)&ns,4);f.write((const char*)&t,8);
        for(int s=0;s<scene_count;++s){
            const long long n=scene_particles[s];
            std::vector<double> X(3*n),V(3*n),Fe(9*n),Jp(n),V0(n),m(n),l(n),mu(n);std::vector<int> valid(n);
            mpm_particle_arrays o{};o.n=n;o.dtype=MPM_F64;o.X=X.data();o.V=V.data();o.Fe=Fe.data();o.Jp=Jp.data();o.V0=V0.data();
            o.mass=m.data();o.lambda0=l.data();o.mu0=mu.data();o.valid=valid.data();
            check(mpm_get_particles(ctx,s,&o),ctx,"mpm_get_particles");
            const int64_t nn=n;f.write((const char*)&nn,8);
            for(auto* v:{&X,&V,&Fe,&Jp,&V0,&m,&l,&mu}) f.write((const char*)v->data(),8*v->size());
            f.write((const char*)valid.data(),4*n);}
        if(!f) throw std::runtime_error("cannot write "+dir+"/checkpoint");
    }

    // Read_Output_Files (MPM_Example.cpp:1065-1079) after the scenes of the test were set
    // up: the full-state checkpoint when the frame has one, else the reference's particle
    // record, which restores X, V, mass and volume and starts every particle with Fe = I,
    // Jp = 1 (as the reference's restart does). The record lists the valid particles only;
    // they take the scene's first slots and any others are marked removed. Returns the
    // simulation time to continue from.
    double Read_Output_Files(int frame)
    {
        const std::string dir=output_directory+"/"+std::to_string(frame);
        std::ifstream c(dir+"/checkpoint",std::ios::binary);
        if(c){
            char magic[8];int32_t ns=0;double t=0;
            c.read(magic,8);c.read((char*)&ns,4);c.read((char*)&t,8);
            if(!c||std::string(magic,8)!="MPMCKPT1"||ns!=scene_count) throw std::runtime_error("bad checkpoint "+dir+"/checkpoint");
            for(int s=0;s<scene_count;++s){
                int64_t n=0;c.read((char*)&n,8);
                if(n!=scene_particles[s]) throw std::runtime_error("checkpoint particle count differs from the test's");
                std::vector<double> X(3*n),V(3*n),Fe(9*n),Jp(n),V0(n),m(n),l(n),mu(n);std::vector<int> valid(n);
                for(auto* v:{&X,&V,&Fe,&Jp,&V0,&m,&l,&mu}) c.read((char*)v->data(),8*v->size());
                c.read((char*)valid.data(),4*n);
                if(!c) throw std::runtime_error("truncated checkpoint "+dir+"/checkpoint");
                mpm_particle_arrays p{};p.n=n;p.dtype=MPM_F64;p.X=X.data();p.V=V.data();p.Fe=Fe.data();p.Jp=Jp.data();p.V0=V0.data();
                p.mass=m.data();p.lambda0=l.data();p.mu0=mu.data();p.valid=valid.data();
                check(mpm_set_particles(ctx,s,&p),ctx,"mpm_set_particles");}
            check(mpm_set_time(ctx,t),ctx,"mpm_set_time");
            return t;}
        for(int s=0;s<scene_count;++s){
            std::ifstream f(dir+"/particles"+(scene_count>1?"_"+std::to_string(s):std::string()),std::ios::binary);
            size_t count=0;f.read((char*)&count,sizeof(count));
            const long long n=scene_particles[s];
            if(!f||(long long)count>n) throw std::runtime_error("cannot read "+dir+"/particles for this test");
            std::vector<float> X(3*n,0.5f),V(3*n,0.f),m(n,0.f),v0(n,0.f),Fe(9*n,0.f),Jp(n,1.f);std::vector<int> valid(n,0);
            for(size_t i=0;i<count;++i){
                f.read((char*)&X[3*i],12);f.read((char*)&V[3*i],12);f.read((char*)&m[i],4);f.read((char*)&v0[i],4);valid[i]=1;}
            if(!f) throw std::runtime_error("truncated "+dir+"/particles");
            for(long long i=0;i<n;++i) for(int k=0;k<3;++k) Fe[9*i+4*k]=1.f;
            mpm_particle_arrays p{};p.n=n;p.dtype=MPM_F32;p.X=X.data();p.V=V.data();p.mass=m.data();p.V0=v0.data();
            p.Fe=Fe.data();p.Jp=Jp.data();p.valid=valid.data();
            check(mpm_set_particles(ctx,s,&p),ctx,"mpm_set_particles");}
        const double t=Time_At_Frame(frame);
        check(mpm_set_time(ctx,t),ctx,"mpm_set_time");
        return t;
    }
};

// MPM_Driver<T,3> (MPM_Driver.cpp:18-116)
class MPM_Driver
{
  public:
    MPM_Example& example;
    double time=0;
    long long substeps=0;
    explicit MPM_Driver(MPM_Example& e):example(e){}

    // MPM_Driver.cpp:18-32. A restart sets up the test's scenes, builds the context and then
    // replaces the particle state with the frame read back.
    void Initialize()
    {
        time=0;
        example.Initialize();
        example.Reset_Grid_Based_Variables();example.Update_Particle_Weights();example.Group_Particles();
        example.Rasterize_Voxels();example.Rasterize();example.Process_Waiting_Particles();
        if(example.restart){
            time=example.Read_Output_Files(example.restart_frame);
            example.current_frame=example.output_number=example.restart_frame;}
    }
    void Execute_Main_Program(){Initialize();Simulate_To_Frame(example.last_frame);}
    // MPM_Driver.cpp:55-80: CFL substeps (fixed_dt>0 replaces the CFL dt) with the same
    // end-of-frame rule.
    // MPM_Driver.cpp:55-80. With a fixed dt the substeps are issued from here, with the
    // same end-of-frame split; in CFL mode the device evaluates the rule before every
    // substep and the whole advance is one call (mpm_advance_to_time).
    void Advance_To_Target_Time(double target_time)
    {
        example.Populate_Simulated_Particles();
        if(example.fixed_dt<=0){
            check(mpm_set_time(example.ctx,time),example.ctx,"mpm_set_time");
            int n=0;
            const mpm_status s=mpm_advance_to_time(example.ctx,target_time,example.cfl,1<<24,&n);
            if(s!=MPM_OK&&s!=MPM_CG_NOT_CONVERGED) check(s,example.ctx,"mpm_advance_to_time");
            check(mpm_get_time(example.ctx,&time),example.ctx,"mpm_get_time");
            substeps+=n;
            return;}
        bool done=false;
        while(!done){
            double dt=example.fixed_dt;
            if(target_time-time<dt*1.001){dt=target_time-time;done=true;}
            else if(target_time-time<2.*dt) dt=(target_time-time)*.5;
            Advance_Step(dt);
            time+=dt;substeps++;}
    }
    void Simulate_To_Frame(int target_frame)
    {
        if(!example.restart) example.Write_Output_Files(example.current_frame);
        while(example.current_frame<target_frame){
            ++example.current_frame;
            Advance_To_Target_Time(example.Time_At_Frame(example.current_frame));
            example.Write_Output_Files(++example.output_number);}
    }
    // MPM_Driver.cpp:103-116, same call order
    void Advance_Step(double dt)
    {
        example.Initialize_SPGrid();example.Reset_Grid_Based_Variables();example.Update_Particle_Weights();
        example.Group_Particles();example.Rasterize_Voxels();example.Rasterize();
        example.Update_Constitutive_Model_State();example.Update_Particle_Velocities_And_Positions(dt);
    }
};

} // namespace mpm_host
