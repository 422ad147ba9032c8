// mpm_3d_main.cpp — command-line driver mirroring mpm_3d/main.cpp:10-32 of the reference:
// parse the options, build the example, run MPM_Driver::Execute_Main_Program, report time.
//   mpm_3d -test_number 101 -last_frame 1 [-dt 1e-4] [-cfl 0.1] [-precision fp32|mixed|fp64]
//          [-seed 0] [-graphs 0|1] [-o dir] [-restart frame] [-threads N (accepted, unused)]
#include "mpm_host.h"

#include <chrono>
#include <cstdlib>
#include <cstring>
#include <iostream>

int main(int argc,char** argv)
{
    using namespace mpm_host;
    auto t0=std::chrono::steady_clock::now();
    MPM_Example example;
    for(int i=1;i<argc;++i){
        const std::string a=argv[i];
        auto next=[&]()->std::string{if(i+1>=argc){std::cerr<<"missing value for "<<a<<"\n";std::exit(2);}return argv[++i];};
        if(a=="-test_number") example.test_number=std::atoi(next().c_str());
        else if(a=="-last_frame") example.last_frame=std::atoi(next().c_str());
        else if(a=="-dt") example.fixed_dt=std::atof(next().c_str());
        else if(a=="-cfl") example.cfl=std::atof(next().c_str());
        else if(a=="-seed") example.seed=std::strtoull(next().c_str(),nullptr,10);
        else if(a=="-graphs") example.config.use_graphs=std::atoi(next().c_str());
        else if(a=="-o"){example.output_directory=next();example.write_output=true;}
        else if(a=="-threads") next();
        else if(a=="-restart"){example.restart=true;example.restart_frame=std::atoi(next().c_str());}
        else if(a=="-precision"){const std::string p=next();
            example.config.precision=p=="fp64"?MPM_PRECISION_FP64:p=="mixed"?MPM_PRECISION_MIXED:MPM_PRECISION_FP32;}
        else{std::cerr<<"unknown option "<<a<<"\n";return 2;}}
    try{
        MPM_Driver driver(example);
        driver.Execute_Main_Program();
        auto t1=std::chrono::steady_clock::now();
        mpm_stats st;mpm_get_stats(example.ctx,0,&st);
        long long np=0;for(long long n:example.scene_particles) np+=n;
        const double sec=std::chrono::duration<double>(t1-t0).count();
        std::cout<<"frames "<<example.last_frame<<" substeps "<<driver.substeps<<" particles "<<np
                 <<" last_cg_iterations "<<st.cg_iterations<<" total_duration "<<sec<<" s\n";
    }catch(const std::exception& e){std::cerr<<e.what()<<"\n";return 1;}
    return 0;
}
