// mpm_capi.cu — the C ABI (include/mpm_gb300.h): context, device memory, the per-substep
// launch sequence (eager, or one CUDA graph per substep whose CG loop is a device-side
// conditional WHILE node), particle upload/download, statistics and timing.
#include "mpm_gb300.h"
#include "mpm_binning.cuh"
#include "mpm_transfer.cuh"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace mpm;

namespace {

enum Phase { PH_KEYS=0, PH_SORT, PH_BIN, PH_P2G, PH_GRID, PH_HESS, PH_CGNODE, PH_G2P, PH_COUNT };
const char* kPhaseNames[PH_COUNT]={"keys","sort","binning","p2g","grid_update","hessian","cg_nodes","g2p"};

struct HostScene {
    mpm_scene_desc desc;
    int nb[3];
    long long block_base,nblocks;
    std::vector<std::pair<long long,long long>> pid_ranges;   // [start,end) of global insertion indices
    long long n_particles;
};

} // namespace

struct mpm_context {
    mpm_config cfg{};
    int num_sms=0;
    cudaStream_t stream=nullptr,stream2=nullptr,stream3=nullptr,stream4=nullptr;
    std::string err;
    std::vector<HostScene> scenes;
    long long total_blocks=0,n_total=0;
    int cur=0;
    bool initialized=false,buffers_ready=false;
    size_t tsize=4;
    // particles
    void* pstate[2]={nullptr,nullptr}; int* pid[2]={nullptr,nullptr}; int* scn[2]={nullptr,nullptr}; void* cache=nullptr;
    // keys[b] start as all ones and are only ever written over [0, n_total), so the sort's
    // final buffer always holds a non-decreasing key array (what incremental binning needs)
    unsigned* keys[2]={nullptr,nullptr}; int* vals[2]={nullptr,nullptr};
    // incremental binning: moved keys and slots (ping-pong for the sort passes) and the
    // per-32-slot moved words
    unsigned* mkeys[2]={nullptr,nullptr}; int* mvals[2]={nullptr,nullptr}; int* manchor=nullptr; uint2* mwords=nullptr;
    int sort_incremental=0;                   // 1: merge the moved slots into the previous order
    // Zeroed once per substep: digit histograms [0,1024), sort tile counters [1024,1028),
    // binning segment counters [1028,1030), incremental key-pass tile counter 1030 and
    // moved count 1031, binning status words from 1280 (work-item counts, then last block
    // heads from bin_heads_off, then active blocks from bin_blocks_off), incremental
    // key-pass status words from inc_status_off, sort status words from sort_status_off.
    unsigned* sortws=nullptr; long long sortws_len=0,bin_heads_off=0,bin_blocks_off=0,inc_status_off=0,sort_status_off=0;
    int* chunk_start=nullptr; long long chunk_cap=0;
    // blocks and nodes
    unsigned* bitmap=nullptr; long long bitmap_words=0;
    int* blockmap=nullptr; int* active_gb=nullptr; int* active_scene=nullptr; long long block_cap=0;
    void *gv=nullptr,*gf=nullptr,*gx=nullptr,*gr=nullptr,*gs=nullptr,*gm=nullptr;
    unsigned char* gproj=nullptr;
    // scenes and solver state
    void* scenes_dev=nullptr; long long* scene_block_base=nullptr;
    CGState* cg=nullptr; SceneAcc* acc=nullptr; SceneAcc* acc2=nullptr; Counters* ctr=nullptr;
    SceneRange* srange=nullptr; ActiveList* alist=nullptr;
    Counters* h_ctr=nullptr; CGState* h_cg=nullptr;
    double* d_dt=nullptr; double last_dt=-1;
    double time=0;                            // simulation clock (seconds)
    FrameState* frame=nullptr; FrameState* h_frame=nullptr;
    void* staging=nullptr; size_t staging_bytes=0;
    int* inv=nullptr;                         // slot of each particle by global insertion index (direct transfers)
    long long order_epoch=0,inv_epoch=-1;     // the particle order changes with every substep; inv follows it
    bool pageable_access=false,host_direct=true;
    // graphs (one per buffer parity)
    cudaGraphExec_t gexec[2]={nullptr,nullptr};
    double graph_dt=0; long long graph_ntotal=-1; bool graph_valid=false;
    long long graph_kernels_outside=0,graph_kernels_body=0;
    // frame graphs of mpm_advance_to_time (one per starting parity)
    cudaGraphExec_t fgexec[2]={nullptr,nullptr};
    bool frame_graph_valid=false; long long frame_kernels_per_substep=0;
    int sort_passes=0;
    int minb_hess=4,minb_p2g=4,minb_g2p=4;   // transfer-kernel occupancy variants
    int xfer_grid=12;                        // transfer-kernel CTAs per SM (grid-stride over work items)
    int node_grid=4;                         // node-kernel (grid update, CG vectors) CTAs per SM
    int hess_warp=HESS_AUTO;                 // Hessian work items per CTA (0), per warp (1), or chosen per launch (2)
    bool use_pdl=true;                       // substep kernels as programmatic dependents
    // timing
    bool timing=false;
    cudaEvent_t ev_pair[2]={nullptr,nullptr};
    double phase_ms[PH_COUNT]={0};
    long long phase_launches[PH_COUNT]={0};
    long long launches=0,substeps=0;
    unsigned long long loop_iters_seen=0;
    // capture-time launch counting
    long long* count_into=nullptr;
};

namespace {

mpm_status fail(mpm_context* c,mpm_status s,const std::string& msg){if(c) c->err=msg;return s;}
#define CUDA_TRY(ctx,call) do{cudaError_t e_=(call);if(e_!=cudaSuccess){return fail(ctx,MPM_CUDA_ERROR,std::string(#call)+": "+cudaGetErrorString(e_));}}while(0)

template<class P> using TT=typename P::T;

// Occupancy variants of the transfer kernels: resident CTAs per SM the register allocation
// is capped for (128-thread CTAs). Chosen per context (tuned on the device).
constexpr int kXferVariants[]={3,4,5,6,8};
template<int V> struct Int{static constexpr int value=V;};
template<class F> void with_minb(int minb,F&& f)
{
    switch(minb){case 3:f(Int<3>{});break;case 5:f(Int<5>{});break;case 6:f(Int<6>{});break;case 8:f(Int<8>{});break;default:f(Int<4>{});}
}

int grid_for(mpm_context* c,int per_sm){return std::max(1,c->num_sms*per_sm);}

// A substep kernel launched on `st` as a programmatic dependent of the kernel before it: it
// may be scheduled while that one drains, and waits for its completion in pdl_enter().
// Phase timing launches plainly, so that the events bracket each phase.
template<class... KA,class... A> void launch_dep(mpm_context* c,void(*k)(KA...),int grid,int block,size_t smem,cudaStream_t st,A&&... a)
{
    cudaLaunchAttribute at[1];
    at[0].id=cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed=1;
    cudaLaunchConfig_t cfg={};
    cfg.gridDim=dim3((unsigned)grid);cfg.blockDim=dim3((unsigned)block);cfg.dynamicSmemBytes=smem;cfg.stream=st;
    cfg.attrs=at;cfg.numAttrs=(c->use_pdl&&!c->timing)?1u:0u;
    cudaLaunchKernelEx(&cfg,k,std::forward<A>(a)...);
}

// ---------- launch bookkeeping ----------
struct PhaseScope {
    mpm_context* c; int ph; cudaStream_t st;
    PhaseScope(mpm_context* c_,int ph_,cudaStream_t st_):c(c_),ph(ph_),st(st_){if(c->timing) cudaEventRecord(c->ev_pair[0],st);}
    ~PhaseScope(){
        if(c->timing){cudaEventRecord(c->ev_pair[1],st);cudaEventSynchronize(c->ev_pair[1]);
            float ms=0;cudaEventElapsedTime(&ms,c->ev_pair[0],c->ev_pair[1]);c->phase_ms[ph]+=ms;}}
};
inline void counted(mpm_context* c,int ph,int n=1)
{
    if(c->count_into) *c->count_into+=n;
    else {c->launches+=n;c->phase_launches[ph]+=n;}
}

// Block bits of a key as the sort passes see them.
unsigned sort_umask(const mpm_context* c){return c->sort_passes>=4?0xFFFFFFFFu:(1u<<(8*c->sort_passes))-1u;}

template<class P> DevState<TT<P>> make_state(mpm_context* c,int parity,double dt)
{
    using T=TT<P>;
    DevState<T> S{};
    S.pcur=(T*)c->pstate[parity];S.pnxt=(T*)c->pstate[parity^1];
    S.pid_cur=c->pid[parity];S.pid_nxt=c->pid[parity^1];
    S.scn_cur=c->scn[parity];S.scn_nxt=c->scn[parity^1];
    S.cache=(T*)c->cache;S.pcap=c->cfg.max_particles;S.n_total=c->n_total;
    const int fin=c->sort_passes&1;   // the sort's final ping-pong buffer
    S.keys=c->keys[fin];S.perm=c->vals[fin];
    S.chunk_start=c->chunk_start;S.chunk_cap=c->chunk_cap;
    S.bitmap=c->bitmap;S.bitmap_words=c->bitmap_words;
    S.blockmap=c->blockmap;S.active_gb=c->active_gb;S.active_scene=c->active_scene;S.block_cap=c->block_cap;
    S.gv=(V4<T>*)c->gv;S.gf=(V4<T>*)c->gf;S.gx=(V4<T>*)c->gx;S.gr=(V4<T>*)c->gr;S.gs=(V4<T>*)c->gs;S.gm=(T*)c->gm;S.gproj=c->gproj;
    S.scenes=(const SceneDev<T>*)c->scenes_dev;S.n_scenes=(int)c->scenes.size();
    S.scene_block_base=c->scene_block_base;
    S.cg=c->cg;S.acc=c->acc;S.acc2=c->acc2;S.ctr=c->ctr;S.srange=c->srange;S.alist=c->alist;
    S.dtp=c->d_dt;S.chunk=c->cfg.chunk;(void)dt;
    return S;
}

// Keys, stable radix sort, work items and active blocks for the current particle buffer.
template<class P> void enqueue_binning(mpm_context* c,cudaStream_t st,const DevState<TT<P>>& S)
{
    const long long n=c->n_total;
    {PhaseScope ps(c,PH_KEYS,st);
        cudaMemsetAsync(c->ctr,0,offsetof(Counters,error),st);
        cudaMemsetAsync(c->bitmap,0,c->bitmap_words*sizeof(unsigned),st);
        cudaMemsetAsync(c->srange,0,sizeof(SceneRange)*c->scenes.size(),st);
        const int g=(int)std::min<long long>((n+256*KEY_ITEMS-1)/(256*KEY_ITEMS),grid_for(c,8));
        const int items=os_items(n);
        const long long num_tiles=(n+(long long)RS_THREADS*items-1)/((long long)RS_THREADS*items);
        cudaMemsetAsync(c->sortws,0,sizeof(unsigned)*(c->sort_status_off+(long long)c->sort_passes*num_tiles*256),st);
        if(c->sort_incremental){
            const int fin=c->sort_passes&1;
            const int gk=(int)std::max<long long>(1,std::min<long long>((n+256*MV_ITEMS-1)/(256*MV_ITEMS),grid_for(c,8)));
            launch_dep(c,k_keys_moved<TT<P>>,gk,MV_THREADS,0,st,S,(const unsigned*)c->keys[fin],c->keys[fin^1],c->mwords,c->sortws,
                       c->sort_passes,sort_umask(c));
            counted(c,PH_KEYS);
            const int gc=(int)std::max<long long>(1,std::min<long long>((n+MC_TILE-1)/MC_TILE,grid_for(c,8)));
            launch_dep(c,k_moved_compact,gc,MC_THREADS,0,st,(const unsigned*)c->keys[fin],(const unsigned*)c->keys[fin^1],c->mwords,n,
                       sort_umask(c),c->sortws+c->inc_status_off,c->sortws+1030,&c->ctr->error,c->mkeys[0],c->vals[fin^1],c->manchor,
                       c->sortws+1031);
            counted(c,PH_KEYS);}
        else{launch_dep(c,k_keys<TT<P>>,std::max(g,1),256,0,st,S,c->keys[0],c->vals[0],c->sortws,c->sort_passes);counted(c,PH_KEYS);}}
    if(c->sort_incremental){PhaseScope ps(c,PH_SORT,st);
        // the moved slots through the same one-sweep passes (their count read on the
        // device; the grid covers all n), then the merge into the sort's final buffer
        const int items=os_items(n);
        const int num_tiles=(int)((n+(long long)RS_THREADS*items-1)/((long long)RS_THREADS*items));
        const int g=std::min(num_tiles,grid_for(c,4));
        const unsigned* m_total=c->sortws+1031;
        for(int p=0;p<c->sort_passes;++p){
            const int a=p&1,b=a^1;
            unsigned* hist=c->sortws+256*p;unsigned* ctrp=c->sortws+4*256+p;
            unsigned* status=c->sortws+c->sort_status_off+(long long)p*num_tiles*256;
            const int* vin=p==0?nullptr:c->mvals[a];     // values: the compaction index
            if(items==RS_ITEMS_SMALL) launch_dep(c,k_onesweep<RS_ITEMS_SMALL>,g,RS_THREADS,0,st,c->mkeys[a],vin,c->mkeys[b],c->mvals[b],n,6+8*p,hist,status,ctrp,num_tiles,&c->ctr->error,m_total);
            else launch_dep(c,k_onesweep<RS_ITEMS>,g,RS_THREADS,0,st,c->mkeys[a],vin,c->mkeys[b],c->mvals[b],n,6+8*p,hist,status,ctrp,num_tiles,&c->ctr->error,m_total);
            counted(c,PH_SORT);}
        // the moved list's passes end in the sort's final parity; the other parity's value
        // buffer is free and takes the sorted ranks
        const int fin=c->sort_passes&1;
        launch_dep(c,k_moved_out,grid_for(c,8),256,0,st,(const unsigned*)c->mkeys[fin],(const int*)c->mvals[fin],(const int*)c->vals[fin^1],
                   (const int*)c->manchor,(const uint2*)c->mwords,m_total,n,c->keys[fin],c->vals[fin],c->mvals[fin^1]);
        counted(c,PH_SORT);
        launch_dep(c,k_merge_unmoved,(int)std::max<long long>(1,std::min<long long>((n+MU_TILE-1)/MU_TILE,grid_for(c,8))),MU_THREADS,0,st,(const unsigned*)c->keys[fin^1],(const uint2*)c->mwords,
                   (const int*)c->mvals[fin^1],m_total,n,c->keys[fin],c->vals[fin]);
        counted(c,PH_SORT);}
    else {PhaseScope ps(c,PH_SORT,st);
        // one-sweep LSD passes over the block bits (above the 6 cell bits); cells inside a
        // block keep their previous (stable) order. sortws: hist[4][256], tile counters at
        // 4*256, status words from 5*256.
        const int items=os_items(n);
        const int num_tiles=(int)((n+(long long)RS_THREADS*items-1)/((long long)RS_THREADS*items));
        const int g=std::min(num_tiles,grid_for(c,4));
        for(int p=0;p<c->sort_passes;++p){
            const int a=p&1,b=a^1;
            const int shift=6+8*p;
            unsigned* hist=c->sortws+256*p;unsigned* ctrp=c->sortws+4*256+p;
            unsigned* status=c->sortws+c->sort_status_off+(long long)p*num_tiles*256;
            const int* vin=p==0?nullptr:c->vals[a];
            if(items==RS_ITEMS_SMALL) launch_dep(c,k_onesweep<RS_ITEMS_SMALL>,g,RS_THREADS,0,st,c->keys[a],vin,c->keys[b],c->vals[b],n,shift,hist,status,ctrp,num_tiles,&c->ctr->error,(const unsigned*)nullptr);
            else launch_dep(c,k_onesweep<RS_ITEMS>,g,RS_THREADS,0,st,c->keys[a],vin,c->keys[b],c->vals[b],n,shift,hist,status,ctrp,num_tiles,&c->ctr->error,(const unsigned*)nullptr);
            counted(c,PH_SORT);}}
    {PhaseScope ps(c,PH_BIN,st);
        const long long nseg=(n+CH_SEG-1)/CH_SEG;
        const int g=(int)std::max<long long>(1,std::min<long long>(nseg,grid_for(c,8)));
        launch_dep(c,k_chunk_heads<TT<P>>,g,CH_THREADS,0,st,S,n,c->cfg.chunk,c->sortws+1280,c->sortws+c->bin_heads_off,c->sortws+1028);counted(c,PH_BIN);
        const long long bseg=(c->bitmap_words+BM_SEG-1)/BM_SEG;
        const int gb=(int)std::max<long long>(1,std::min<long long>(bseg,grid_for(c,8)));
        launch_dep(c,k_bitmap_index<TT<P>>,gb,SC_THREADS,0,st,S,c->sortws+c->bin_blocks_off,c->sortws+1029);counted(c,PH_BIN);
        launch_dep(c,k_clear_nodes<TT<P>>,grid_for(c,8),256,0,st,S);counted(c,PH_BIN);}
}

int max_cg_iters(mpm_context* c){int m=0;for(auto& s:c->scenes) m=std::max(m,s.desc.cg_max_iters);return m;}

// One Hessian product in the context's form: work items per CTA, per warp, or chosen per launch.
template<class P,bool FROM_X> void launch_hessian(mpm_context* c,cudaStream_t st,const DevState<TT<P>>& S2)
{
    with_minb(c->minb_hess,[&](auto m){
        // the automatic form's threshold: the warps resident at this occupancy variant
        const long long warp_min=(long long)c->num_sms*decltype(m)::value*(XFER_THREADS/32);
        launch_dep(c,k_hessian<P,FROM_X,decltype(m)::value>,grid_for(c,c->xfer_grid),XFER_THREADS,hess_kernel_smem_bytes<TT<P>>(),st,S2,c->hess_warp,warp_min);});
}

template<class P> void enqueue_cg_body(mpm_context* c,cudaStream_t st,const DevState<TT<P>>& S2,unsigned long long cond,int use_cond)
{
    {PhaseScope ps(c,PH_HESS,st);
        launch_hessian<P,false>(c,st,S2);counted(c,PH_HESS);}
    {PhaseScope ps(c,PH_CGNODE,st);
        launch_dep(c,k_cg_q<P>,grid_for(c,c->node_grid),NODE_THREADS,0,st,S2);counted(c,PH_CGNODE);
        launch_dep(c,k_cg_update<P>,grid_for(c,c->node_grid),NODE_THREADS,0,st,S2,cond,use_cond,max_cg_iters(c)+1);counted(c,PH_CGNODE);}
}

// Everything of one substep before the CG loop. Returns the state with swapped buffers.
template<class P> DevState<TT<P>> enqueue_pre(mpm_context* c,cudaStream_t st,int parity,double dt,unsigned long long cond,int use_cond,int stop_after)
{
    DevState<TT<P>> S=make_state<P>(c,parity,dt);
    enqueue_binning<P>(c,st,S);
    {PhaseScope ps(c,PH_P2G,st);
        with_minb(c->minb_p2g,[&](auto m){launch_dep(c,k_p2g<P,decltype(m)::value>,grid_for(c,c->xfer_grid),XFER_THREADS,p2g_smem_bytes<TT<P>>(c->cfg.chunk),st,S);});counted(c,PH_P2G);}
    DevState<TT<P>> S2=make_state<P>(c,parity^1,dt);
    {PhaseScope ps(c,PH_GRID,st);launch_dep(c,k_grid_update<TT<P>>,grid_for(c,c->node_grid),NODE_THREADS,0,st,S2);counted(c,PH_GRID);}
    if(stop_after==1||stop_after==2) return S2;
    {PhaseScope ps(c,PH_HESS,st);
        launch_hessian<P,true>(c,st,S2);counted(c,PH_HESS);}
    {PhaseScope ps(c,PH_CGNODE,st);launch_dep(c,k_cg_start<P>,grid_for(c,c->node_grid),NODE_THREADS,0,st,S2,cond,use_cond);counted(c,PH_CGNODE);}
    return S2;
}
template<class P> void enqueue_post(mpm_context* c,cudaStream_t st,const DevState<TT<P>>& S2)
{
    PhaseScope ps(c,PH_G2P,st);
    with_minb(c->minb_g2p,[&](auto m){launch_dep(c,k_g2p<TT<P>,decltype(m)::value>,grid_for(c,c->xfer_grid),XFER_THREADS,0,st,S2);});counted(c,PH_G2P);
}

__global__ void k_set_dt(double* p,double v){*p=v;}
// One decoupled look-back of the binning scans (chained_prefix) for segment 1 of a zeroed
// status array: segment 0 never publishes, so the wait gives up after spin_limit polls and
// sets ERR_SORT_WAIT.
__global__ void __launch_bounds__(32) k_lookback_selftest(unsigned* status,unsigned* error,int spin_limit)
{
    chained_prefix(status,1,1u,error,spin_limit);
}
void set_dt(mpm_context* c,double dt)
{
    if(dt==c->last_dt) return;
    k_set_dt<<<1,1,0,c->stream>>>(c->d_dt,dt);c->launches++;
    c->last_dt=dt;
}


// Eager substep: host-driven CG loop that reads the device's loop flag every iteration.
template<class P> mpm_status substep_eager(mpm_context* c,double dt,int stop_after,bool dt_on_device=false)
{
    cudaStream_t st=c->stream;
    if(!dt_on_device) set_dt(c,dt);
    DevState<TT<P>> S2=enqueue_pre<P>(c,st,c->cur,dt,0,0,stop_after);
    if(stop_after==1||stop_after==2){return MPM_OK;}
    const int cap=max_cg_iters(c)+1;
    for(int it=0;it<cap;++it){
        CUDA_TRY(c,cudaMemcpyAsync(&c->h_ctr->any_active,&c->ctr->any_active,sizeof(int),cudaMemcpyDeviceToHost,st));
        CUDA_TRY(c,cudaStreamSynchronize(st));
        if(!c->h_ctr->any_active) break;
        enqueue_cg_body<P>(c,st,S2,0,0);}
    if(stop_after==3) return MPM_OK;
    enqueue_post<P>(c,st,S2);
    c->cur^=1;c->order_epoch++;
    c->substeps++;
    if(!dt_on_device) c->time+=dt;
    return MPM_OK;
}

// Creates a conditional handle on the graph that `st` is capturing into.
mpm_status capture_handle(mpm_context* c,cudaStream_t st,unsigned dflt,cudaGraphConditionalHandle* h)
{
    cudaStreamCaptureStatus cs;cudaGraph_t g=nullptr;
    CUDA_TRY(c,cudaStreamGetCaptureInfo(st,&cs,nullptr,&g,nullptr,nullptr,nullptr));
    CUDA_TRY(c,cudaGraphConditionalHandleCreate(h,g,dflt,cudaGraphCondAssignDefault));
    return MPM_OK;
}
// Adds a conditional node (WHILE or IF on `h`) at the capture point of `st`, makes it the
// point `st` continues from, and starts capturing its body on `st_body`.
mpm_status capture_conditional(mpm_context* c,cudaStream_t st,cudaStream_t st_body,cudaGraphConditionalHandle h,cudaGraphConditionalNodeType type)
{
    cudaStreamCaptureStatus cs;cudaGraph_t g=nullptr;const cudaGraphNode_t* deps=nullptr;size_t ndeps=0;
    CUDA_TRY(c,cudaStreamGetCaptureInfo(st,&cs,nullptr,&g,&deps,nullptr,&ndeps));
    cudaGraphNodeParams cp{};
    cp.type=cudaGraphNodeTypeConditional;
    cp.conditional.handle=h;cp.conditional.type=type;cp.conditional.size=1;
    cudaGraphNode_t cnode;
    CUDA_TRY(c,cudaGraphAddNode(&cnode,g,deps,nullptr,ndeps,&cp));
    CUDA_TRY(c,cudaStreamUpdateCaptureDependencies(st,&cnode,nullptr,1,cudaStreamSetCaptureDependencies));
    CUDA_TRY(c,cudaStreamBeginCaptureToGraph(st_body,cp.conditional.phGraph_out[0],nullptr,nullptr,0,cudaStreamCaptureModeThreadLocal));
    return MPM_OK;
}
mpm_status end_body_capture(mpm_context* c,cudaStream_t st_body)
{
    cudaGraph_t tmp;
    CUDA_TRY(c,cudaStreamEndCapture(st_body,&tmp));
    return MPM_OK;
}
// One whole substep (the CG loop a WHILE node) into the graph `st` is capturing; the CG
// body is captured on `st_body`. Kernel counts go to *outside and *body.
template<class P> mpm_status capture_substep(mpm_context* c,cudaStream_t st,cudaStream_t st_body,int parity,double dt,long long* outside,long long* body)
{
    cudaGraphConditionalHandle h;
    mpm_status s=capture_handle(c,st,0,&h);if(s!=MPM_OK) return s;
    c->count_into=outside;
    DevState<TT<P>> S2=enqueue_pre<P>(c,st,parity,dt,(unsigned long long)h,1,0);
    s=capture_conditional(c,st,st_body,h,cudaGraphCondTypeWhile);if(s!=MPM_OK){c->count_into=nullptr;return s;}
    c->count_into=body;
    enqueue_cg_body<P>(c,st_body,S2,(unsigned long long)h,1);
    s=end_body_capture(c,st_body);
    c->count_into=outside;
    if(s==MPM_OK) enqueue_post<P>(c,st,S2);
    c->count_into=nullptr;
    return s;
}

template<class P> mpm_status build_graphs(mpm_context* c,double dt)
{
    for(int parity=0;parity<2;++parity){
        if(c->gexec[parity]){cudaGraphExecDestroy(c->gexec[parity]);c->gexec[parity]=nullptr;}
        cudaStream_t st=c->stream;
        long long outside=0,body=0;
        CUDA_TRY(c,cudaStreamBeginCapture(st,cudaStreamCaptureModeThreadLocal));
        mpm_status s=capture_substep<P>(c,st,c->stream2,parity,dt,&outside,&body);
        cudaGraph_t full=nullptr;
        const cudaError_t ee=cudaStreamEndCapture(st,&full);
        if(s!=MPM_OK){if(full) cudaGraphDestroy(full);return s;}
        if(ee!=cudaSuccess) return fail(c,MPM_CUDA_ERROR,std::string("cudaStreamEndCapture: ")+cudaGetErrorString(ee));
        cudaError_t e=cudaGraphInstantiate(&c->gexec[parity],full,0);
        cudaGraphDestroy(full);
        if(e!=cudaSuccess) return fail(c,MPM_CUDA_ERROR,std::string("cudaGraphInstantiate: ")+cudaGetErrorString(e));
        c->graph_kernels_outside=outside;c->graph_kernels_body=body;}
    c->graph_dt=dt;c->graph_ntotal=c->n_total;c->graph_valid=true;
    return MPM_OK;
}

// The frame graph of mpm_advance_to_time for a starting parity: a WHILE loop whose body is
// two substeps (parities p and p^1, so the buffers alternate), each preceded by k_cfl; the
// second one sits in an IF node that k_cfl of the first opens only when the advance goes
// on, and k_frame_cond closes the loop once a substep has ended the advance.
template<class P> mpm_status build_frame_graphs(mpm_context* c)
{
    if(!c->stream3&&cudaStreamCreateWithFlags(&c->stream3,cudaStreamNonBlocking)!=cudaSuccess) return fail(c,MPM_CUDA_ERROR,"stream");
    if(!c->stream4&&cudaStreamCreateWithFlags(&c->stream4,cudaStreamNonBlocking)!=cudaSuccess) return fail(c,MPM_CUDA_ERROR,"stream");
    for(int parity=0;parity<2;++parity){
        if(c->fgexec[parity]){cudaGraphExecDestroy(c->fgexec[parity]);c->fgexec[parity]=nullptr;}
        cudaStream_t st=c->stream,s2=c->stream2,s3=c->stream3,s4=c->stream4;
        long long outside=0,body=0,extra=0;
        CUDA_TRY(c,cudaStreamBeginCapture(st,cudaStreamCaptureModeThreadLocal));
        mpm_status s=MPM_OK;
        int open=0;   // body captures in progress (s2, s3)
        cudaGraphConditionalHandle h_outer,h_more;
        const int gcfl=grid_for(c,4);
        do{
            if((s=capture_handle(c,st,1,&h_outer))!=MPM_OK) break;
            if((s=capture_conditional(c,st,s2,h_outer,cudaGraphCondTypeWhile))!=MPM_OK) break;
            open=1;
            if((s=capture_handle(c,s2,0,&h_more))!=MPM_OK) break;
            k_cfl<TT<P>><<<gcfl,NODE_THREADS,0,s2>>>(make_state<P>(c,parity,0.),c->frame,c->d_dt,(unsigned long long)h_more,1);extra++;
            if((s=capture_substep<P>(c,s2,s3,parity,0.,&outside,&body))!=MPM_OK) break;
            if((s=capture_conditional(c,s2,s3,h_more,cudaGraphCondTypeIf))!=MPM_OK) break;
            open=2;
            k_cfl<TT<P>><<<gcfl,NODE_THREADS,0,s3>>>(make_state<P>(c,parity^1,0.),c->frame,c->d_dt,0ull,0);
            long long o2=0,b2=0;
            if((s=capture_substep<P>(c,s3,s4,parity^1,0.,&o2,&b2))!=MPM_OK) break;
            if((s=end_body_capture(c,s3))!=MPM_OK) break;
            open=1;
            k_frame_cond<<<1,32,0,s2>>>(c->frame,(unsigned long long)h_outer);
            if((s=end_body_capture(c,s2))!=MPM_OK) break;
            open=0;
        }while(false);
        if(open>=2){cudaGraph_t t;cudaStreamEndCapture(s3,&t);}
        if(open>=1){cudaGraph_t t;cudaStreamEndCapture(s2,&t);}
        cudaGraph_t full=nullptr;
        const cudaError_t ee=cudaStreamEndCapture(st,&full);
        if(s==MPM_OK&&ee!=cudaSuccess) s=fail(c,MPM_CUDA_ERROR,std::string("frame graph capture: ")+cudaGetErrorString(ee));
        if(s==MPM_OK){
            const cudaError_t e=cudaGraphInstantiate(&c->fgexec[parity],full,0);
            if(e!=cudaSuccess) s=fail(c,MPM_CUDA_ERROR,std::string("frame graph instantiate: ")+cudaGetErrorString(e));}
        if(full) cudaGraphDestroy(full);
        if(s!=MPM_OK) return s;
        c->frame_kernels_per_substep=outside+extra;c->graph_kernels_body=body;}
    c->frame_graph_valid=true;c->graph_ntotal=c->n_total;
    return MPM_OK;
}

template<class P> mpm_status substep_graph(mpm_context* c,double dt)
{
    set_dt(c,dt);
    if(!c->graph_valid||c->graph_ntotal!=c->n_total){
        mpm_status s=build_graphs<P>(c,dt);if(s!=MPM_OK) return s;}
    CUDA_TRY(c,cudaGraphLaunch(c->gexec[c->cur],c->stream));
    c->launches+=c->graph_kernels_outside;
    c->cur^=1;c->order_epoch++;c->substeps++;c->time+=dt;
    return MPM_OK;
}

// Reads the counters and solver state back and turns error bits into a status.
mpm_status collect_status(mpm_context* c)
{
    CUDA_TRY(c,cudaMemcpyAsync(c->h_ctr,c->ctr,sizeof(Counters),cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(c->h_cg,c->cg,sizeof(CGState)*c->scenes.size(),cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    CUDA_TRY(c,cudaGetLastError());
    const unsigned e=c->h_ctr->error;
    // loop trips of graph launches are counted on the device
    const unsigned long long trips=c->h_ctr->total_trips;
    if(trips>c->loop_iters_seen){c->launches+=(long long)(trips-c->loop_iters_seen)*c->graph_kernels_body;}
    c->loop_iters_seen=trips;
    if(e&ERR_CAPACITY) return fail(c,MPM_CAPACITY,"capacity exceeded (particles, work items or node blocks); raise max_blocks/max_particles");
    if(e&ERR_NONFINITE){
        const unsigned b=c->h_ctr->bad_scene1;
        return fail(c,MPM_NONFINITE,std::string("non-finite particle position")+
                    (b?" (highest scene index with one: "+std::to_string((int)b-1)+")":std::string()));}
    if(e&ERR_OUT_OF_GRID) return fail(c,MPM_BAD_ARG,"particle outside the grid; it was removed");
    if(e&ERR_SORT_WAIT) return fail(c,MPM_CUDA_ERROR,"sort look-back wait exceeded its limit");
    if(e&ERR_CG_NOT_CONVERGED) return MPM_CG_NOT_CONVERGED;
    return MPM_OK;
}

template<class T> void fill_scene_dev(const HostScene& h,long long pid_base,SceneDev<T>& d)
{
    std::memset(&d,0,sizeof(d));
    const mpm_scene_desc& s=h.desc;
    for(int a=0;a<3;++a){d.counts[a]=s.counts[a];d.nb[a]=h.nb[a];d.dx[a]=(T)(1.0/(double)s.counts[a]);d.inv_dx[a]=(T)s.counts[a];d.gravity[a]=(T)s.gravity[a];}
    d.block_base=h.block_base;d.pid_base=pid_base;d.flip=(T)s.flip;
    d.plastic=s.plastic;d.hardening=(T)s.hardening;d.cy=(T)s.compression_yield;d.sy=(T)s.stretching_yield;
    d.hmax=(T)std::min(s.hardening_max,(double)FLT_MAX);
    d.project=s.project;d.n_barriers=s.n_barriers;
    for(int b=0;b<s.n_barriers;++b){for(int a=0;a<3;++a){d.bn[b][a]=(T)s.barriers[b].normal[a];d.bs[b][a]=(T)s.barriers[b].surface[a];}
        d.bmu[b]=(T)s.barriers[b].mu;d.bsticky[b]=s.barriers[b].sticky;}
    d.cg_abs_tol=s.cg_abs_tol;d.cg_rel_tol=s.cg_rel_tol;d.cg_max_iters=s.cg_max_iters;d.cg_min_iters=s.cg_min_iters;
    d.eos=s.material==MPM_MATERIAL_EOS_FLUID;d.bulk=(T)s.bulk_modulus;d.eos_gamma=(T)s.eos_gamma;
}

mpm_status ensure_staging(mpm_context* c,size_t bytes)
{
    if(bytes<=c->staging_bytes) return MPM_OK;
    if(c->staging){cudaStreamSynchronize(c->stream);cudaFree(c->staging);c->staging=nullptr;c->staging_bytes=0;}
    CUDA_TRY(c,cudaMalloc(&c->staging,bytes));
    c->staging_bytes=bytes;
    return MPM_OK;
}

// ---------- particle ingest / egress kernels ----------
// Source arrays live in `staging` back to back in this order (each n rows): X(3) V(3)
// mass lambda0 mu0 Fe(9) Jp V0; absent optional arrays are flagged in `have`.
struct InLayout { long long n; int have_fe,have_jp,have_v0,have_mass,have_lam,have_mu; };
template<class T,class Tin> __global__ void k_ingest(const Tin* __restrict__ src,InLayout L,T* state,int* pid,int* scn,long long pcap,
                                                     long long slot0,long long pid0,int scene,int mode)
{
    // mode 0: append to slots slot0.. ; mode 1: overwrite the slots whose pid is in [pid0, pid0+n)
    const long long n=L.n;
    const Tin* X=src;const Tin* V=X+3*n;const Tin* M=V+3*n;const Tin* LA=M+n;const Tin* MU=LA+n;const Tin* FE=MU+n;const Tin* JP=FE+9*n;const Tin* VV=JP+n;
    const long long total=mode==0?n:slot0;   // in mode 1 slot0 carries n_total
    for(long long k=blockIdx.x*(long long)blockDim.x+threadIdx.x;k<total;k+=(long long)gridDim.x*blockDim.x){
        long long i,j;
        if(mode==0){j=k;i=slot0+k;pid[i]=(int)(pid0+k);scn[i]=scene;}
        else{i=k;j=(long long)pid[i]-pid0;if(j<0||j>=n) continue;scn[i]=scene;}
        for(int a=0;a<3;++a){state[(FX+a)*pcap+i]=(T)X[3*j+a];state[(FV+a)*pcap+i]=(T)V[3*j+a];}
        if(L.have_mass) state[FM*pcap+i]=(T)M[j];
        if(L.have_lam) state[FLAM0*pcap+i]=(T)LA[j];
        if(L.have_mu) state[FMU0*pcap+i]=(T)MU[j];
        for(int k2=0;k2<9;++k2) if(L.have_fe||mode==0) state[(FF+k2)*pcap+i]=L.have_fe?(T)FE[9*j+k2]:((k2%4==0)?T(1):T(0));
        if(L.have_jp||mode==0) state[FJP*pcap+i]=L.have_jp?(T)JP[j]:T(1);
        if(L.have_v0||mode==0) state[FV0*pcap+i]=L.have_v0?(T)VV[j]:T(0);}
}
template<class T,class Tout> __global__ void k_egress(const T* __restrict__ state,const int* __restrict__ pid,const int* __restrict__ scn,long long pcap,
                                                      long long n_total,long long pid0,long long n,int scene,Tout* dst)
{
    Tout* X=dst;Tout* V=X+3*n;Tout* FE=V+3*n;Tout* JP=FE+9*n;Tout* VV=JP+n;Tout* M=VV+n;Tout* VAL=M+n;Tout* LA=VAL+n;Tout* MU=LA+n;
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<n_total;i+=(long long)gridDim.x*blockDim.x){
        const long long j=(long long)pid[i]-pid0;if(j<0||j>=n) continue;
        const int s=scn[i];const int home=s>=0?s:-s-1;if(home!=scene) continue;
        for(int a=0;a<3;++a){X[3*j+a]=(Tout)state[(FX+a)*pcap+i];V[3*j+a]=(Tout)state[(FV+a)*pcap+i];}
        for(int k=0;k<9;++k) FE[9*j+k]=(Tout)state[(FF+k)*pcap+i];
        JP[j]=(Tout)state[FJP*pcap+i];VV[j]=(Tout)state[FV0*pcap+i];M[j]=(Tout)state[FM*pcap+i];VAL[j]=(Tout)(s>=0?1:0);
        LA[j]=(Tout)state[FLAM0*pcap+i];MU[j]=(Tout)state[FMU0*pcap+i];}
}

// New particles (source rows as in k_ingest) written into given slots of the scene, reset as
// Allocate_Particle resets them (MPM_Example.cpp:959-975, the particle's Initialize()):
// Fe NULL = identity, Jp NULL = 1, V0 NULL = 0 (computed by the volume pass).
template<class T,class Tin> __global__ void k_place(const Tin* __restrict__ src,InLayout L,const int* __restrict__ slots,T* state,int* scn,
                                                    long long pcap,int scene)
{
    const long long n=L.n;
    const Tin* X=src;const Tin* V=X+3*n;const Tin* M=V+3*n;const Tin* LA=M+n;const Tin* MU=LA+n;const Tin* FE=MU+n;const Tin* JP=FE+9*n;const Tin* VV=JP+n;
    for(long long j=blockIdx.x*(long long)blockDim.x+threadIdx.x;j<n;j+=(long long)gridDim.x*blockDim.x){
        const long long i=slots[j];
        for(int a=0;a<3;++a){state[(FX+a)*pcap+i]=(T)X[3*j+a];state[(FV+a)*pcap+i]=(T)V[3*j+a];}
        state[FM*pcap+i]=(T)M[j];state[FLAM0*pcap+i]=(T)LA[j];state[FMU0*pcap+i]=(T)MU[j];
        for(int k=0;k<9;++k) state[(FF+k)*pcap+i]=L.have_fe?(T)FE[9*j+k]:((k%4==0)?T(1):T(0));
        state[FJP*pcap+i]=L.have_jp?(T)JP[j]:T(1);
        state[FV0*pcap+i]=L.have_v0?(T)VV[j]:T(0);
        scn[i]=scene;}
}
// valid[j] == 0 marks the j-th of n particles appended at slot0 as removed (a reserve slot).
__global__ void k_valid_range(const int* __restrict__ valid,long long slot0,long long n,int* scn,int scene)
{
    for(long long j=blockIdx.x*(long long)blockDim.x+threadIdx.x;j<n;j+=(long long)gridDim.x*blockDim.x)
        scn[slot0+j]=valid[j]?scene:-(scene+1);
}

// Direct transfers, for hosts where the GPU reads and writes the caller's arrays in place
// (pinned memory, or any memory where the device uses the host page tables). inv[j] is the
// slot of the scene's j-th particle (insertion order), so host arrays are streamed in
// order and only the device side is gathered.
__global__ void k_slot_map(const int* __restrict__ pid,long long n_total,long long pid0,long long n,int* __restrict__ inv)
{
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<n_total;i+=(long long)gridDim.x*blockDim.x){
        const long long j=(long long)pid[i]-pid0;
        if(j>=0&&j<n) inv[j]=(int)i;}
}
// The slot of every particle by global insertion index, rebuilt once after the particle
// order changed (a substep, mpm_initialize, a restore) and shared by the transfers of all
// scenes until the next change: scene transfers index it from their first insertion index.
static void ensure_slot_map(mpm_context* c)
{
    if(c->inv_epoch==c->order_epoch) return;
    k_slot_map<<<std::max(1,c->num_sms*4),256,0,c->stream>>>(c->pid[c->cur],c->n_total,0,c->n_total,c->inv);
    c->launches++;
    c->inv_epoch=c->order_epoch;
}
// One host array of n*ncomp elements and the state field of its first component.
// Consecutive threads take consecutive host elements (the host side is streamed in order;
// only the device side is gathered through inv).
struct HostField { void* p; int ncomp; int field; };
struct HostFields { HostField f[9]; int count; };
template<class T,class Th> __global__ void k_ingest_direct(HostFields H,long long n,const int* __restrict__ inv,T* state,int* scn,long long pcap,int scene)
{
    const long long t0=blockIdx.x*(long long)blockDim.x+threadIdx.x,stride=(long long)gridDim.x*blockDim.x;
    for(long long j=t0;j<n;j+=stride) scn[inv[j]]=scene;
    for(int k=0;k<H.count;++k){
        const Th* src=(const Th*)H.f[k].p;const int nc=H.f[k].ncomp;const long long base=(long long)H.f[k].field*pcap;
        for(long long e=t0;e<n*nc;e+=stride){
            const long long j=e/nc;const int a=(int)(e-j*nc);
            state[base+a*pcap+inv[j]]=(T)src[e];}}
}
template<class T,class Th> __global__ void k_egress_direct(const T* __restrict__ state,const int* __restrict__ scn,long long pcap,const int* __restrict__ inv,
                                                           long long n,HostFields H,int* valid)
{
    const long long t0=blockIdx.x*(long long)blockDim.x+threadIdx.x,stride=(long long)gridDim.x*blockDim.x;
    for(int k=0;k<H.count;++k){
        Th* dst=(Th*)H.f[k].p;const int nc=H.f[k].ncomp;const long long base=(long long)H.f[k].field*pcap;
        for(long long e=t0;e<n*nc;e+=stride){
            const long long j=e/nc;const int a=(int)(e-j*nc);
            dst[e]=(Th)state[base+a*pcap+inv[j]];}}
    if(valid) for(long long j=t0;j<n;j+=stride) valid[j]=scn[inv[j]]>=0?1:0;
}
// valid[j] == 0 marks the scene's j-th particle removed (scene id -(s+1)), else simulated.
__global__ void k_apply_valid(const int* __restrict__ valid,const int* __restrict__ inv,long long n,int* scn,int scene)
{
    for(long long j=blockIdx.x*(long long)blockDim.x+threadIdx.x;j<n;j+=(long long)gridDim.x*blockDim.x)
        scn[inv[j]]=valid[j]?scene:-(scene+1);
}
static HostFields host_fields(void* X,void* V,void* mass,void* lam,void* mu,void* Fe,void* Jp,void* V0)
{
    HostFields H{};
    auto add=[&](void* p,int nc,int field){if(p){H.f[H.count].p=p;H.f[H.count].ncomp=nc;H.f[H.count].field=field;H.count++;}};
    add(X,3,FX);add(V,3,FV);add(mass,1,FM);add(lam,1,FLAM0);add(mu,1,FMU0);add(Fe,9,FF);add(Jp,1,FJP);add(V0,1,FV0);
    return H;
}

template<class T> __global__ void k_interior_export(DevState<T> S,int scene,long long cap,int* coords,double* m,double* v,double* vs,unsigned long long* count)
{
    const long long nn=(long long)min(S.ctr->n_active,(unsigned)S.block_cap)*64;
    for(long long n=blockIdx.x*(long long)blockDim.x+threadIdx.x;n<nn;n+=(long long)gridDim.x*blockDim.x){
        const int blk=(int)(n>>6);if(S.active_scene[blk]!=scene) continue;
        const T mm=S.gm[n];if(!(mm>T(0))) continue;
        const unsigned long long k=atomicAdd(count,1ull);if((long long)k>=cap) continue;
        const SceneDev<T>& sc=S.scenes[scene];
        long long lb=(long long)S.active_gb[blk]-sc.block_base;
        const int bx=(int)(lb%sc.nb[0]);lb/=sc.nb[0];const int by=(int)(lb%sc.nb[1]),bz=(int)(lb/sc.nb[1]);
        const int l=(int)(n&63);
        if(coords){coords[3*k]=4*bx+(l&3)-4;coords[3*k+1]=4*by+((l>>2)&3)-4;coords[3*k+2]=4*bz+(l>>4)-4;}
        if(m) m[k]=(double)mm;
        const V4<T> a=S.gv[n],b=S.gx[n];
        if(v){v[3*k]=a.x;v[3*k+1]=a.y;v[3*k+2]=a.z;}
        if(vs){vs[3*k]=b.x;vs[3*k+1]=b.y;vs[3*k+2]=b.z;}}
}
// Particle bounding box of a scene (X +- 2/counts clamped to [0,1]) as float bits with an
// order-preserving map, for the Dirichlet count of Rasterize_Voxels.
__device__ __forceinline__ unsigned long long ord_bits(double x){long long b=__double_as_longlong(x);return b>=0?(unsigned long long)b^0x8000000000000000ull:~(unsigned long long)b;}
template<class T> __global__ void k_bbox(DevState<T> S,int scene,unsigned long long* mn,unsigned long long* mx)
{
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<S.n_total;i+=(long long)gridDim.x*blockDim.x){
        if(S.scn_cur[i]!=scene) continue;
        const SceneDev<T>& sc=S.scenes[scene];
        for(int a=0;a<3;++a){const T x=S.pcur[(FX+a)*S.pcap+i];const T dd=(T)2./(T)sc.counts[a];
            atomicMin(&mn[a],ord_bits((double)(x-dd)));atomicMax(&mx[a],ord_bits((double)(x+dd)));}}
}
template<class T> __global__ void k_count_in_box(DevState<T> S,int scene,int lo0,int lo1,int lo2,int hi0,int hi1,int hi2,unsigned long long* count)
{
    const long long nn=(long long)min(S.ctr->n_active,(unsigned)S.block_cap)*64;
    for(long long n=blockIdx.x*(long long)blockDim.x+threadIdx.x;n<nn;n+=(long long)gridDim.x*blockDim.x){
        const int blk=(int)(n>>6);if(S.active_scene[blk]!=scene) continue;
        if(!(S.gm[n]>T(0))) continue;
        const SceneDev<T>& sc=S.scenes[scene];
        long long lb=(long long)S.active_gb[blk]-sc.block_base;
        const int bx=(int)(lb%sc.nb[0]);lb/=sc.nb[0];const int by=(int)(lb%sc.nb[1]),bz=(int)(lb/sc.nb[1]);
        const int l=(int)(n&63);
        const int c0=4*bx+(l&3)-4,c1=4*by+((l>>2)&3)-4,c2=4*bz+(l>>4)-4;
        if(c0>=lo0&&c0<=hi0&&c1>=lo1&&c1<=hi1&&c2>=lo2&&c2<=hi2) atomicAdd(count,1ull);}
}
template<class T> __global__ void k_vmax(DevState<T> S,int scene,unsigned long long* out)
{
    double m=0.;
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<S.n_total;i+=(long long)gridDim.x*blockDim.x){
        if(S.scn_cur[i]!=scene) continue;
        T s=T(0);for(int a=0;a<3;++a){const T v=S.pcur[(FV+a)*S.pcap+i];s+=v*v;}
        m=fmax(m,(double)s);}
    for(int o=16;o>0;o>>=1) m=fmax(m,__shfl_xor_sync(0xffffffffu,m,o));
    if((threadIdx.x&31)==0&&m>0.) atomicMax(out,(unsigned long long)__double_as_longlong(m));
}

// The private tiles of the FP64 P2G exceed the default 48 KB of dynamic shared memory.
template<class P> void set_smem_limits()
{
    for(int v:kXferVariants) with_minb(v,[&](auto m){
        cudaFuncSetAttribute(k_p2g<P,decltype(m)::value>,cudaFuncAttributeMaxDynamicSharedMemorySize,p2g_smem_bytes<TT<P>>(4096));
        cudaFuncSetAttribute(k_hessian<P,false,decltype(m)::value>,cudaFuncAttributeMaxDynamicSharedMemorySize,hess_kernel_smem_bytes<TT<P>>());
        cudaFuncSetAttribute(k_hessian<P,true,decltype(m)::value>,cudaFuncAttributeMaxDynamicSharedMemorySize,hess_kernel_smem_bytes<TT<P>>());});
}

template<class P> mpm_status alloc_buffers(mpm_context* c)
{
    set_smem_limits<P>();
    // A warp per Hessian work item pays off once there are several work items (about 400
    // particles each) per resident warp: from about 6M particles on a 152-SM GB300.
    using T=TT<P>;
    const long long pc=c->cfg.max_particles;
    // scenes: block ranges
    long long base=0;
    std::vector<long long> bases;
    for(auto& s:c->scenes){s.block_base=base;bases.push_back(base);base+=s.nblocks;}
    bases.push_back(base);
    c->total_blocks=base;
    if(base*64>=(long long)KEY_SENTINEL) return fail(c,MPM_CAPACITY,"scenes too large for 32-bit cell keys");
    int bits=1;while((1LL<<bits)<=base) bits++;     // bits of the block id (the key's upper part)
    c->sort_passes=(bits+7)/8;
    c->bitmap_words=(base+31)/32;
    c->block_cap=c->cfg.max_blocks>0?c->cfg.max_blocks:std::min<long long>(base,std::max<long long>(4096,pc/16));
    c->chunk_cap=c->block_cap+pc/c->cfg.chunk+16;
    const long long nodes=c->block_cap*64;
    auto M=[&](void** p,size_t bytes)->cudaError_t{return cudaMalloc(p,std::max<size_t>(bytes,16));};
    {   const long long nseg=(pc+CH_SEG-1)/CH_SEG+1,bseg=(c->bitmap_words+BM_SEG-1)/BM_SEG+1;
        c->bin_heads_off=1280+nseg;
        c->bin_blocks_off=c->bin_heads_off+nseg;
        c->inc_status_off=c->bin_blocks_off+bseg;
        c->sort_status_off=((c->inc_status_off+(pc+MC_TILE-1)/MC_TILE+1+255)/256)*256;
        c->sortws_len=c->sort_status_off+4LL*((pc+(long long)RS_THREADS*RS_ITEMS_SMALL-1)/((long long)RS_THREADS*RS_ITEMS_SMALL))*256;}
    CUDA_TRY(c,M((void**)&c->sortws,sizeof(unsigned)*c->sortws_len));
    CUDA_TRY(c,M((void**)&c->chunk_start,sizeof(int)*c->chunk_cap));
    CUDA_TRY(c,M((void**)&c->bitmap,sizeof(unsigned)*c->bitmap_words));
    CUDA_TRY(c,M((void**)&c->blockmap,sizeof(int)*base));
    CUDA_TRY(c,M((void**)&c->active_gb,sizeof(int)*c->block_cap));
    CUDA_TRY(c,M((void**)&c->active_scene,sizeof(int)*c->block_cap));
    CUDA_TRY(c,M(&c->gv,sizeof(V4<T>)*nodes));CUDA_TRY(c,M(&c->gf,sizeof(V4<T>)*nodes));
    CUDA_TRY(c,M(&c->gx,sizeof(V4<T>)*nodes));CUDA_TRY(c,M(&c->gr,sizeof(V4<T>)*nodes));
    CUDA_TRY(c,M(&c->gs,sizeof(V4<T>)*nodes));CUDA_TRY(c,M(&c->gm,sizeof(T)*nodes));
    CUDA_TRY(c,M((void**)&c->gproj,nodes));
    CUDA_TRY(c,M((void**)&c->scene_block_base,sizeof(long long)*bases.size()));
    CUDA_TRY(c,cudaMemcpy(c->scene_block_base,bases.data(),sizeof(long long)*bases.size(),cudaMemcpyHostToDevice));
    std::vector<SceneDev<T>> sd(c->scenes.size());
    long long pidb=0;
    for(size_t i=0;i<c->scenes.size();++i){fill_scene_dev<T>(c->scenes[i],pidb,sd[i]);pidb+=c->scenes[i].n_particles;}
    CUDA_TRY(c,cudaMemcpy(c->scenes_dev,sd.data(),sizeof(SceneDev<T>)*sd.size(),cudaMemcpyHostToDevice));
    CUDA_TRY(c,cudaMemset(c->acc,0,sizeof(SceneAcc)*c->cfg.max_scenes));
    CUDA_TRY(c,cudaMemset(c->acc2,0,sizeof(SceneAcc)*c->cfg.max_scenes));
    CUDA_TRY(c,cudaMemset(c->cg,0,sizeof(CGState)*c->cfg.max_scenes));
    c->buffers_ready=true;
    return MPM_OK;
}

// The grid build of the current particles and the first-touch volumes of those whose V0
// is not positive (Rasterize + Process_Waiting_Particles, MPM_Example.cpp:520-542,
// 827-840); the particles end up permuted into block order in the other buffer.
template<class P> void enqueue_volume_pass(mpm_context* c)
{
    cudaStream_t st=c->stream;
    DevState<TT<P>> S=make_state<P>(c,c->cur,0.0);
    // always the full sort: before the first grid build the previous keys are all ones, so
    // every particle would count as moved
    const int inc=c->sort_incremental;c->sort_incremental=0;
    enqueue_binning<P>(c,st,S);
    c->sort_incremental=inc;
    k_permute<TT<P>><<<grid_for(c,4),256,0,st>>>(S);counted(c,PH_P2G);
    DevState<TT<P>> S2=make_state<P>(c,c->cur^1,0.0);
    k_p2g_mass<TT<P>><<<grid_for(c,c->xfer_grid),XFER_THREADS,0,st>>>(S2);counted(c,PH_P2G);
    k_init_volume<TT<P>><<<grid_for(c,c->xfer_grid),XFER_THREADS,0,st>>>(S2);counted(c,PH_P2G);
    c->cur^=1;c->order_epoch++;
}

template<class P> mpm_status initialize_impl(mpm_context* c)
{
    if(c->scenes.empty()||c->n_total==0) return fail(c,MPM_NOT_READY,"no scenes or particles");
    if(!c->buffers_ready){mpm_status s=alloc_buffers<P>(c);if(s!=MPM_OK) return s;}
    CUDA_TRY(c,cudaMemsetAsync(c->ctr,0,sizeof(Counters),c->stream));
    enqueue_volume_pass<P>(c);
    c->initialized=true;
    return collect_status(c);
}

template<class P> mpm_status advance_impl(mpm_context* c,int k,double dt,int stop_after)
{
    if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
    if(!(dt>0.)) return fail(c,MPM_BAD_ARG,"dt must be positive");
    CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),c->stream));
    for(int i=0;i<k;++i){
        mpm_status s;
        if(stop_after==0&&c->cfg.use_graphs&&!c->timing) s=substep_graph<P>(c,dt);
        else s=substep_eager<P>(c,dt,stop_after);
        if(s!=MPM_OK) return s;}
    return collect_status(c);
}

template<class F> auto dispatch(mpm_context* c,F&& f)
{
    if(c->cfg.precision==MPM_PRECISION_FP32) return f(PrecFP32{});
    if(c->cfg.precision==MPM_PRECISION_MIXED) return f(PrecMixed{});
    return f(PrecFP64{});
}

bool bad_scene(mpm_context* c,int scene){return !c||scene<0||scene>=(int)c->scenes.size();}

} // namespace

extern "C" {

const char* mpm_status_string(mpm_status s)
{
    switch(s){
        case MPM_OK: return "ok";
        case MPM_CG_NOT_CONVERGED: return "CG not converged";
        case MPM_NONFINITE: return "non-finite state";
        case MPM_CAPACITY: return "capacity exceeded";
        case MPM_BAD_ARG: return "bad argument";
        case MPM_CUDA_ERROR: return "CUDA error";
        case MPM_NOT_READY: return "not ready";}
    return "unknown";
}

void mpm_default_config(mpm_config* cfg)
{
    if(!cfg) return;
    std::memset(cfg,0,sizeof(*cfg));
    cfg->precision=MPM_PRECISION_FP32;cfg->device=0;cfg->use_graphs=1;cfg->max_scenes=64;
    cfg->max_particles=1<<20;cfg->max_blocks=0;cfg->chunk=1024;
}

mpm_status mpm_create(const mpm_config* cfg,mpm_context** out)
{
    if(!cfg||!out) return MPM_BAD_ARG;
    *out=nullptr;
    mpm_config c0=*cfg;
    if(c0.precision<0||c0.precision>2||c0.max_scenes<1||c0.max_scenes>MPM_MAX_SCENES||c0.max_particles<1||c0.max_particles>((1LL<<31)-1))
        return MPM_BAD_ARG;
    if(c0.chunk==0) c0.chunk=1024;
    if(c0.chunk<32||c0.chunk>4096) return MPM_BAD_ARG;
    mpm_context* c=new mpm_context();
    c->cfg=c0;
    c->tsize=c0.precision==MPM_PRECISION_FP64?8:4;
    auto bail=[&](mpm_status s){mpm_destroy(c);return s;};
    if(cudaSetDevice(c0.device)!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    cudaDeviceProp prop;
    if(cudaGetDeviceProperties(&prop,c0.device)!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    c->num_sms=prop.multiProcessorCount;
    {int v=0;if(cudaDeviceGetAttribute(&v,cudaDevAttrPageableMemoryAccess,c0.device)==cudaSuccess) c->pageable_access=v!=0;}
    if(const char* v=std::getenv("MPM_HOST_DIRECT")) c->host_direct=std::strcmp(v,"0")!=0;   // "0": always stage host arrays
    if(const char* v=std::getenv("MPM_PDL")) c->use_pdl=std::strcmp(v,"0")!=0;               // "0": plain stream order
    if(const char* v=std::getenv("MPM_HESSIAN_WARP")) c->hess_warp=std::min(2,std::max(0,std::atoi(v)));  // form of the Hessian product
    if(c0.precision==MPM_PRECISION_FP64){c->minb_hess=c->minb_p2g=c->minb_g2p=3;}
    if(const char* v=std::getenv("MPM_XFER_BLOCKS")){   // "hessian,p2g,g2p" occupancy variants (tuning)
        int a=0,b=0,d=0,r=0,g=0;const int k=std::sscanf(v,"%d,%d,%d,%d,%d",&a,&b,&d,&r,&g);
        if(k>=3){c->minb_hess=a;c->minb_p2g=b;c->minb_g2p=d;}(void)r;if(k>=5&&g>0) c->xfer_grid=g;}
    if(const char* v=std::getenv("MPM_SORT_INCREMENTAL")) c->sort_incremental=std::atoi(v)?1:0;
    if(cudaStreamCreateWithFlags(&c->stream,cudaStreamNonBlocking)!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    if(cudaStreamCreateWithFlags(&c->stream2,cudaStreamNonBlocking)!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    if(cudaEventCreate(&c->ev_pair[0])!=cudaSuccess||cudaEventCreate(&c->ev_pair[1])!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    const long long pc=c0.max_particles;const size_t ts=c->tsize;
    bool ok=true;
    for(int b=0;b<2;++b){
        ok&=cudaMalloc(&c->pstate[b],ts*NB_FIELDS*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->pid[b],sizeof(int)*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->scn[b],sizeof(int)*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->keys[b],sizeof(unsigned)*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->vals[b],sizeof(int)*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->mkeys[b],sizeof(unsigned)*pc)==cudaSuccess;
        ok&=cudaMalloc((void**)&c->mvals[b],sizeof(int)*pc)==cudaSuccess;
        ok&=ok&&cudaMemset(c->keys[b],0xFF,sizeof(unsigned)*pc)==cudaSuccess;}
    ok&=cudaMalloc((void**)&c->mwords,sizeof(uint2)*(pc/32+1))==cudaSuccess;
    ok&=cudaMalloc((void**)&c->manchor,sizeof(int)*pc)==cudaSuccess;
    ok&=cudaMalloc(&c->cache,ts*NC_FIELDS*pc)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->inv,sizeof(int)*std::max<long long>(pc,1))==cudaSuccess;
    const size_t sdsz=ts==8?sizeof(SceneDev<double>):sizeof(SceneDev<float>);
    ok&=cudaMalloc(&c->scenes_dev,sdsz*c0.max_scenes)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->cg,sizeof(CGState)*c0.max_scenes)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->acc,sizeof(SceneAcc)*c0.max_scenes)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->acc2,sizeof(SceneAcc)*c0.max_scenes)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->ctr,sizeof(Counters))==cudaSuccess;
    ok&=cudaMalloc((void**)&c->srange,sizeof(SceneRange)*c0.max_scenes)==cudaSuccess;
    ok&=cudaMalloc((void**)&c->alist,sizeof(ActiveList))==cudaSuccess;
    ok&=cudaMalloc((void**)&c->d_dt,sizeof(double))==cudaSuccess;
    ok&=cudaMalloc((void**)&c->frame,sizeof(FrameState))==cudaSuccess;
    ok&=cudaMallocHost((void**)&c->h_frame,sizeof(FrameState))==cudaSuccess;
    ok&=cudaMallocHost((void**)&c->h_ctr,sizeof(Counters))==cudaSuccess;
    ok&=cudaMallocHost((void**)&c->h_cg,sizeof(CGState)*c0.max_scenes)==cudaSuccess;
    if(!ok) return bail(MPM_CUDA_ERROR);
    if(cudaMemset(c->ctr,0,sizeof(Counters))!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    if(cudaMemset(c->alist,0,sizeof(ActiveList))!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    if(cudaMemset(c->srange,0,sizeof(SceneRange)*c0.max_scenes)!=cudaSuccess) return bail(MPM_CUDA_ERROR);
    *out=c;
    return MPM_OK;
}

mpm_status mpm_destroy(mpm_context* c)
{
    if(!c) return MPM_OK;
    if(c->stream) cudaStreamSynchronize(c->stream);
    for(int p=0;p<2;++p){if(c->gexec[p]) cudaGraphExecDestroy(c->gexec[p]);if(c->fgexec[p]) cudaGraphExecDestroy(c->fgexec[p]);}
    void* bufs[]={c->pstate[0],c->pstate[1],c->pid[0],c->pid[1],c->scn[0],c->scn[1],c->cache,c->keys[0],c->keys[1],c->vals[0],c->vals[1],
                  c->sortws,c->chunk_start,c->bitmap,c->blockmap,c->active_gb,c->active_scene,c->gv,c->gf,c->gx,c->gr,c->gs,c->gm,c->gproj,
                  c->scenes_dev,c->scene_block_base,c->cg,c->acc,c->acc2,c->ctr,c->staging,c->d_dt,c->frame,c->inv,
                  c->srange,c->alist,c->mkeys[0],c->mkeys[1],c->mvals[0],c->mvals[1],c->mwords,c->manchor};
    for(void* p:bufs) if(p) cudaFree(p);
    if(c->h_ctr) cudaFreeHost(c->h_ctr);
    if(c->h_cg) cudaFreeHost(c->h_cg);
    if(c->h_frame) cudaFreeHost(c->h_frame);
    for(auto& e:c->ev_pair) if(e) cudaEventDestroy(e);
    if(c->stream) cudaStreamDestroy(c->stream);
    if(c->stream2) cudaStreamDestroy(c->stream2);
    if(c->stream3) cudaStreamDestroy(c->stream3);
    if(c->stream4) cudaStreamDestroy(c->stream4);
    delete c;
    return MPM_OK;
}

const char* mpm_last_error(const mpm_context* c){return c?c->err.c_str():"null context";}

mpm_status mpm_add_scene(mpm_context* c,const mpm_scene_desc* d,int* scene_id)
{
    if(!c||!d) return MPM_BAD_ARG;
    if(c->buffers_ready) return fail(c,MPM_NOT_READY,"scenes must be added before mpm_initialize");
    if((int)c->scenes.size()>=c->cfg.max_scenes) return fail(c,MPM_CAPACITY,"max_scenes reached");
    for(int a=0;a<3;++a) if(d->counts[a]<4||d->counts[a]%4||d->counts[a]>4096) return fail(c,MPM_BAD_ARG,"counts must be multiples of 4 in [4,4096]");
    if(d->n_barriers<0||d->n_barriers>MPM_MAX_BARRIERS) return fail(c,MPM_BAD_ARG,"n_barriers out of range");
    if(d->material!=MPM_MATERIAL_SNOW&&d->material!=MPM_MATERIAL_EOS_FLUID) return fail(c,MPM_BAD_ARG,"unknown material");
    if(d->material==MPM_MATERIAL_EOS_FLUID&&!(d->bulk_modulus>0.&&d->eos_gamma>=1.)) return fail(c,MPM_BAD_ARG,"EOS fluid needs bulk_modulus > 0 and eos_gamma >= 1");
    HostScene h;h.desc=*d;h.n_particles=0;h.block_base=0;
    h.nblocks=1;for(int a=0;a<3;++a){h.nb[a]=d->counts[a]/4+2;h.nblocks*=h.nb[a];}
    c->scenes.push_back(h);
    if(scene_id) *scene_id=(int)c->scenes.size()-1;
    return MPM_OK;
}

static size_t elem_size(int dtype){return dtype==MPM_F64?8:4;}

// Whether kernels may read or write the caller's array in place: always where the device
// uses the host page tables (pageable memory access), else only for pinned host memory
// whose device address is the host address.
static bool host_direct_ok(mpm_context* c,const void* p)
{
    if(!p||c->pageable_access) return true;
    cudaPointerAttributes a{};
    if(cudaPointerGetAttributes(&a,p)!=cudaSuccess){cudaGetLastError();return false;}
    return a.type==cudaMemoryTypeHost&&a.devicePointer==p;
}
static bool arrays_direct_ok(mpm_context* c,const mpm_particle_arrays* p)
{
    if(!c->host_direct) return false;
    const void* ptrs[]={p->X,p->V,p->mass,p->lambda0,p->mu0,p->Fe,p->Jp,p->V0,p->valid};
    for(const void* q:ptrs) if(!host_direct_ok(c,q)) return false;
    return true;
}

// `sync`: wait for the copy before returning (a batched call waits once for all scenes;
// only the in-place path, which needs no staging buffer, skips the wait).
static mpm_status upload(mpm_context* c,int scene,const mpm_particle_arrays* p,int mode,bool sync=true)
{
    if(bad_scene(c,scene)||!p||p->n<=0||!p->X||!p->V) return fail(c,MPM_BAD_ARG,"bad particle arrays");
    if(p->dtype!=MPM_F32&&p->dtype!=MPM_F64) return fail(c,MPM_BAD_ARG,"dtype");
    if(mode==0&&(!p->mass||!p->lambda0||!p->mu0)) return fail(c,MPM_BAD_ARG,"mass, lambda0 and mu0 are required");
    const long long n=p->n;const size_t es=elem_size(p->dtype);
    HostScene& hs=c->scenes[scene];
    if(mode==0){
        if(c->n_total+n>c->cfg.max_particles) return fail(c,MPM_CAPACITY,"max_particles exceeded");
        if(c->buffers_ready) return fail(c,MPM_NOT_READY,"particles must be added before mpm_initialize");
        // positions must lie inside [0,1]^3 (the reference removes particles outside its cell domain)
        for(long long i=0;i<n;++i) for(int a=0;a<3;++a){
            const double x=p->dtype==MPM_F64?((const double*)p->X)[3*i+a]:((const float*)p->X)[3*i+a];
            if(!(x>=0.&&x<=1.)) return fail(c,MPM_BAD_ARG,"particle position outside [0,1]^3");}}
    else if(n!=hs.n_particles) return fail(c,MPM_BAD_ARG,"mpm_set_particles needs the scene's particle count");
    if(mode==1&&arrays_direct_ok(c,p)){
        if(hs.pid_ranges.size()!=1) return fail(c,MPM_BAD_ARG,"scene particles were added in several batches");
        const long long pid0=hs.pid_ranges[0].first;
        cudaStream_t sm=c->stream;
        const int g=std::max(1,grid_for(c,4));
        ensure_slot_map(c);
        const int* inv=c->inv+pid0;
        const HostFields H=host_fields(p->X,p->V,p->mass,p->lambda0,p->mu0,p->Fe,p->Jp,p->V0);
        void* state=c->pstate[c->cur];
        if(c->cfg.precision==MPM_PRECISION_FP64){
            if(p->dtype==MPM_F64) k_ingest_direct<double,double><<<g,256,0,sm>>>(H,n,inv,(double*)state,c->scn[c->cur],c->cfg.max_particles,scene);
            else k_ingest_direct<double,float><<<g,256,0,sm>>>(H,n,inv,(double*)state,c->scn[c->cur],c->cfg.max_particles,scene);}
        else{
            if(p->dtype==MPM_F64) k_ingest_direct<float,double><<<g,256,0,sm>>>(H,n,inv,(float*)state,c->scn[c->cur],c->cfg.max_particles,scene);
            else k_ingest_direct<float,float><<<g,256,0,sm>>>(H,n,inv,(float*)state,c->scn[c->cur],c->cfg.max_particles,scene);}
        c->launches++;
        if(p->valid){k_apply_valid<<<g,256,0,sm>>>(p->valid,inv,n,c->scn[c->cur],scene);c->launches++;}
        CUDA_TRY(c,cudaGetLastError());
        if(sync) CUDA_TRY(c,cudaStreamSynchronize(sm));
        return MPM_OK;}
    mpm_status s=ensure_staging(c,es*n*20+sizeof(int)*n+16);if(s!=MPM_OK) return s;
    char* st=(char*)c->staging;
    cudaStream_t sm=c->stream;
    auto put=[&](const void* src,long long off,long long cnt)->cudaError_t{if(!src) return cudaSuccess;return cudaMemcpyAsync(st+off*es,src,cnt*es,cudaMemcpyHostToDevice,sm);};
    CUDA_TRY(c,put(p->X,0,3*n));CUDA_TRY(c,put(p->V,3*n,3*n));CUDA_TRY(c,put(p->mass,6*n,n));
    CUDA_TRY(c,put(p->lambda0,7*n,n));CUDA_TRY(c,put(p->mu0,8*n,n));CUDA_TRY(c,put(p->Fe,9*n,9*n));
    CUDA_TRY(c,put(p->Jp,18*n,n));CUDA_TRY(c,put(p->V0,19*n,n));
    InLayout L{n,p->Fe!=nullptr,p->Jp!=nullptr,p->V0!=nullptr,p->mass!=nullptr,p->lambda0!=nullptr,p->mu0!=nullptr};
    long long pid0;
    if(mode==0){pid0=c->n_total;}
    else{if(hs.pid_ranges.size()!=1) return fail(c,MPM_BAD_ARG,"scene particles were added in several batches");pid0=hs.pid_ranges[0].first;}
    const int g=std::max(1,grid_for(c,4));
    const long long slot0=mode==0?c->n_total:c->n_total;
    const bool f64=c->cfg.precision==MPM_PRECISION_FP64;
    void* state=c->pstate[c->cur];
    if(f64){if(p->dtype==MPM_F64) k_ingest<double,double><<<g,256,0,sm>>>((const double*)st,L,(double*)state,c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,slot0,pid0,scene,mode);
            else k_ingest<double,float><<<g,256,0,sm>>>((const float*)st,L,(double*)state,c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,slot0,pid0,scene,mode);}
    else{if(p->dtype==MPM_F64) k_ingest<float,double><<<g,256,0,sm>>>((const double*)st,L,(float*)state,c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,slot0,pid0,scene,mode);
         else k_ingest<float,float><<<g,256,0,sm>>>((const float*)st,L,(float*)state,c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,slot0,pid0,scene,mode);}
    c->launches++;
    if(mode==0&&p->valid){
        int* vdev=(int*)(st+((es*n*20+15)&~(size_t)15));
        CUDA_TRY(c,cudaMemcpyAsync(vdev,p->valid,sizeof(int)*n,cudaMemcpyHostToDevice,sm));
        k_valid_range<<<g,256,0,sm>>>(vdev,slot0,n,c->scn[c->cur],scene);c->launches++;}
    if(mode==1&&p->valid){
        int* vdev=(int*)(st+((es*n*20+15)&~(size_t)15));
        CUDA_TRY(c,cudaMemcpyAsync(vdev,p->valid,sizeof(int)*n,cudaMemcpyHostToDevice,sm));
        ensure_slot_map(c);
        k_apply_valid<<<g,256,0,sm>>>(vdev,c->inv+pid0,n,c->scn[c->cur],scene);c->launches++;}
    CUDA_TRY(c,cudaGetLastError());
    if(mode==0){
        if(!hs.pid_ranges.empty()&&hs.pid_ranges.back().second==pid0) hs.pid_ranges.back().second+=n;
        else hs.pid_ranges.push_back({pid0,pid0+n});
        hs.n_particles+=n;c->n_total+=n;c->graph_valid=false;c->frame_graph_valid=false;c->order_epoch++;}
    CUDA_TRY(c,cudaStreamSynchronize(sm));
    return MPM_OK;
}

mpm_status mpm_add_particles(mpm_context* c,int scene,const mpm_particle_arrays* p){return upload(c,scene,p,0);}
mpm_status mpm_set_particles(mpm_context* c,int scene,const mpm_particle_arrays* p){return upload(c,scene,p,1);}
mpm_status mpm_set_particles_batch(mpm_context* c,int count,const int* scenes,const mpm_particle_arrays* arrays)
{
    if(!c||count<0||(count>0&&(!scenes||!arrays))) return MPM_BAD_ARG;
    for(int k=0;k<count;++k){
        // in place (host arrays the device can read): queued without a wait; else one call
        const bool direct=!bad_scene(c,scenes[k])&&arrays_direct_ok(c,&arrays[k]);
        const mpm_status s=upload(c,scenes[k],&arrays[k],1,!direct);
        if(s!=MPM_OK){cudaStreamSynchronize(c->stream);return s;}}
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    return MPM_OK;
}

mpm_status mpm_allocate_particles(mpm_context* c,int scene,const mpm_particle_arrays* p,int* ids)
{
    if(bad_scene(c,scene)||!p||p->n<=0||!p->X||!p->V||!p->mass||!p->lambda0||!p->mu0) return fail(c,MPM_BAD_ARG,"bad particle arrays");
    if(p->dtype!=MPM_F32&&p->dtype!=MPM_F64) return fail(c,MPM_BAD_ARG,"dtype");
    if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
    const HostScene& hs=c->scenes[scene];
    if(hs.pid_ranges.size()!=1) return fail(c,MPM_BAD_ARG,"scene particles were added in several batches");
    const long long n=p->n;const size_t es=elem_size(p->dtype);
    auto elem=[&](const void* a,long long k)->double{return p->dtype==MPM_F64?((const double*)a)[k]:(double)((const float*)a)[k];};
    bool need_volume=!p->V0;
    for(long long i=0;i<n;++i){
        for(int a=0;a<3;++a){const double x=elem(p->X,3*i+a);if(!(x>=0.&&x<=1.)) return fail(c,MPM_BAD_ARG,"particle position outside [0,1]^3");}
        if(p->V0&&!(elem(p->V0,i)>0.)) need_volume=true;}
    // the scene's removed particles, lowest insertion index first
    const long long nt=c->n_total;
    std::vector<int> pid(nt),scn(nt);
    CUDA_TRY(c,cudaMemcpyAsync(pid.data(),c->pid[c->cur],sizeof(int)*nt,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(scn.data(),c->scn[c->cur],sizeof(int)*nt,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    std::vector<std::pair<int,int>> freed;
    for(long long i=0;i<nt;++i) if(scn[i]==-(scene+1)) freed.push_back({pid[i],(int)i});
    if((long long)freed.size()<n) return fail(c,MPM_CAPACITY,"the scene has fewer removed particles than requested "
                                              "(reserve slots with mpm_add_particles and valid = 0)");
    std::partial_sort(freed.begin(),freed.begin()+n,freed.end());
    std::vector<int> slots(n);
    for(long long k=0;k<n;++k) slots[k]=freed[k].second;
    const size_t data_bytes=(es*n*20+15)&~(size_t)15;
    mpm_status s=ensure_staging(c,data_bytes+sizeof(int)*n);if(s!=MPM_OK) return s;
    char* st=(char*)c->staging;cudaStream_t sm=c->stream;
    auto put=[&](const void* src,long long off,long long cnt)->cudaError_t{if(!src) return cudaSuccess;return cudaMemcpyAsync(st+off*es,src,cnt*es,cudaMemcpyHostToDevice,sm);};
    CUDA_TRY(c,put(p->X,0,3*n));CUDA_TRY(c,put(p->V,3*n,3*n));CUDA_TRY(c,put(p->mass,6*n,n));
    CUDA_TRY(c,put(p->lambda0,7*n,n));CUDA_TRY(c,put(p->mu0,8*n,n));CUDA_TRY(c,put(p->Fe,9*n,9*n));
    CUDA_TRY(c,put(p->Jp,18*n,n));CUDA_TRY(c,put(p->V0,19*n,n));
    int* dslots=(int*)(st+data_bytes);
    CUDA_TRY(c,cudaMemcpyAsync(dslots,slots.data(),sizeof(int)*n,cudaMemcpyHostToDevice,sm));
    InLayout L{n,p->Fe!=nullptr,p->Jp!=nullptr,p->V0!=nullptr,1,1,1};
    const int g=std::max(1,grid_for(c,4));
    void* state=c->pstate[c->cur];
    if(c->cfg.precision==MPM_PRECISION_FP64){
        if(p->dtype==MPM_F64) k_place<double,double><<<g,256,0,sm>>>((const double*)st,L,dslots,(double*)state,c->scn[c->cur],c->cfg.max_particles,scene);
        else k_place<double,float><<<g,256,0,sm>>>((const float*)st,L,dslots,(double*)state,c->scn[c->cur],c->cfg.max_particles,scene);}
    else{
        if(p->dtype==MPM_F64) k_place<float,double><<<g,256,0,sm>>>((const double*)st,L,dslots,(float*)state,c->scn[c->cur],c->cfg.max_particles,scene);
        else k_place<float,float><<<g,256,0,sm>>>((const float*)st,L,dslots,(float*)state,c->scn[c->cur],c->cfg.max_particles,scene);}
    c->launches++;
    CUDA_TRY(c,cudaGetLastError());
    CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),sm));
    if(need_volume){
        dispatch(c,[&](auto pp){enqueue_volume_pass<decltype(pp)>(c);return 0;});}
    if(ids) for(long long k=0;k<n;++k) ids[k]=(int)(freed[k].first-hs.pid_ranges[0].first);
    return collect_status(c);
}

mpm_status mpm_initialize(mpm_context* c)
{
    if(!c) return MPM_BAD_ARG;
    for(auto& s:c->scenes) if(s.pid_ranges.size()>1) return fail(c,MPM_BAD_ARG,"add each scene's particles in one contiguous batch");
    return dispatch(c,[&](auto p){return initialize_impl<decltype(p)>(c);});
}

mpm_status mpm_advance_steps(mpm_context* c,int k,double dt)
{
    if(!c||k<0) return MPM_BAD_ARG;
    return dispatch(c,[&](auto p){return advance_impl<decltype(p)>(c,k,dt,0);});
}
mpm_status mpm_advance_step(mpm_context* c,double dt){return mpm_advance_steps(c,1,dt);}

mpm_status mpm_advance_step_partial(mpm_context* c,double dt,int stop_after)
{
    if(!c||stop_after<0||stop_after>3) return MPM_BAD_ARG;
    const int cur=c->cur;
    mpm_status s=dispatch(c,[&](auto p){return advance_impl<decltype(p)>(c,1,dt,stop_after);});
    if(stop_after!=0) c->cur=cur;   // particle state untouched: the old buffer is still current
    return s;
}

mpm_status mpm_max_particle_velocity(mpm_context* c,int scene,double* vmax)
{
    if(bad_scene(c,scene)||!vmax||!c->initialized) return MPM_BAD_ARG;
    return dispatch(c,[&](auto p)->mpm_status{
        using P=decltype(p);
        DevState<TT<P>> S=make_state<P>(c,c->cur,0.0);
        unsigned long long* tmp=nullptr;
        CUDA_TRY(c,cudaMalloc(&tmp,8));
        CUDA_TRY(c,cudaMemsetAsync(tmp,0,8,c->stream));
        k_vmax<TT<P>><<<grid_for(c,4),256,0,c->stream>>>(S,scene,tmp);c->launches++;
        unsigned long long h=0;
        CUDA_TRY(c,cudaMemcpyAsync(&h,tmp,8,cudaMemcpyDeviceToHost,c->stream));
        CUDA_TRY(c,cudaStreamSynchronize(c->stream));
        cudaFree(tmp);
        double v2;std::memcpy(&v2,&h,8);*vmax=std::sqrt(v2);
        return MPM_OK;});
}

static mpm_status download(mpm_context* c,int scene,mpm_particle_arrays* out,bool sync);
mpm_status mpm_get_particles(mpm_context* c,int scene,mpm_particle_arrays* out){return download(c,scene,out,true);}
mpm_status mpm_get_particles_batch(mpm_context* c,int count,const int* scenes,mpm_particle_arrays* arrays)
{
    if(!c||count<0||(count>0&&(!scenes||!arrays))) return MPM_BAD_ARG;
    for(int k=0;k<count;++k){
        const bool direct=!bad_scene(c,scenes[k])&&arrays_direct_ok(c,&arrays[k]);
        const mpm_status s=download(c,scenes[k],&arrays[k],!direct);
        if(s!=MPM_OK){cudaStreamSynchronize(c->stream);return s;}}
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    return MPM_OK;
}
// `sync`: as for upload; only the in-place path skips the wait.
static mpm_status download(mpm_context* c,int scene,mpm_particle_arrays* out,bool sync)
{
    if(bad_scene(c,scene)||!out) return MPM_BAD_ARG;
    const HostScene& hs=c->scenes[scene];
    const long long n=hs.n_particles;
    if(out->n<n) return fail(c,MPM_BAD_ARG,"output arrays too small");
    if(n==0) return MPM_OK;
    const size_t es=elem_size(out->dtype);
    const long long pid0=hs.pid_ranges.empty()?0:hs.pid_ranges[0].first;
    cudaStream_t sm=c->stream;
    if(hs.pid_ranges.size()==1&&arrays_direct_ok(c,out)){
        const int g=grid_for(c,4);
        ensure_slot_map(c);
        const int* inv=c->inv+pid0;
        const HostFields H=host_fields(out->X,out->V,out->mass,out->lambda0,out->mu0,out->Fe,out->Jp,out->V0);
        dispatch(c,[&](auto p){
            using T=TT<decltype(p)>;
            if(out->dtype==MPM_F64) k_egress_direct<T,double><<<g,256,0,sm>>>((const T*)c->pstate[c->cur],c->scn[c->cur],c->cfg.max_particles,inv,n,H,out->valid);
            else k_egress_direct<T,float><<<g,256,0,sm>>>((const T*)c->pstate[c->cur],c->scn[c->cur],c->cfg.max_particles,inv,n,H,out->valid);
            return 0;});
        c->launches++;
        CUDA_TRY(c,cudaGetLastError());
        if(sync) CUDA_TRY(c,cudaStreamSynchronize(sm));
        return MPM_OK;}
    mpm_status s=ensure_staging(c,es*n*21+16);if(s!=MPM_OK) return s;
    dispatch(c,[&](auto p){
        using T=TT<decltype(p)>;
        const int g=grid_for(c,4);
        if(out->dtype==MPM_F64) k_egress<T,double><<<g,256,0,sm>>>((const T*)c->pstate[c->cur],c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,c->n_total,pid0,n,scene,(double*)c->staging);
        else k_egress<T,float><<<g,256,0,sm>>>((const T*)c->pstate[c->cur],c->pid[c->cur],c->scn[c->cur],c->cfg.max_particles,c->n_total,pid0,n,scene,(float*)c->staging);
        c->launches++;return 0;});
    char* st=(char*)c->staging;
    auto get=[&](void* dst,long long off,long long cnt)->cudaError_t{if(!dst) return cudaSuccess;return cudaMemcpyAsync(dst,st+off*es,cnt*es,cudaMemcpyDeviceToHost,sm);};
    CUDA_TRY(c,get(out->X,0,3*n));CUDA_TRY(c,get(out->V,3*n,3*n));CUDA_TRY(c,get(out->Fe,6*n,9*n));
    CUDA_TRY(c,get(out->Jp,15*n,n));CUDA_TRY(c,get(out->V0,16*n,n));CUDA_TRY(c,get(out->mass,17*n,n));
    CUDA_TRY(c,get(out->lambda0,19*n,n));CUDA_TRY(c,get(out->mu0,20*n,n));
    std::vector<char> valid;
    if(out->valid){valid.resize(n*es);CUDA_TRY(c,cudaMemcpyAsync(valid.data(),st+18*n*es,n*es,cudaMemcpyDeviceToHost,sm));}
    CUDA_TRY(c,cudaStreamSynchronize(sm));
    if(out->valid) for(long long i=0;i<n;++i) out->valid[i]=es==8?(int)((double*)valid.data())[i]:(int)((float*)valid.data())[i];
    CUDA_TRY(c,cudaGetLastError());
    return MPM_OK;
}

mpm_status mpm_get_stats(mpm_context* c,int scene,mpm_stats* out)
{
    if(bad_scene(c,scene)||!out) return MPM_BAD_ARG;
    std::memset(out,0,sizeof(*out));
    out->n_particles=c->scenes[scene].n_particles;out->substeps=c->substeps;
    if(!c->initialized){out->gpu_launches=c->launches;return MPM_OK;}
    CUDA_TRY(c,cudaMemcpyAsync(c->h_cg,c->cg,sizeof(CGState)*c->scenes.size(),cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(c->h_ctr,c->ctr,sizeof(Counters),cudaMemcpyDeviceToHost,c->stream));
    // valid particles and active blocks of this scene
    std::vector<int> scn(c->n_total),ascn;
    CUDA_TRY(c,cudaMemcpyAsync(scn.data(),c->scn[c->cur],sizeof(int)*c->n_total,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    const long long na=std::min<long long>(c->h_ctr->n_active,c->block_cap);
    ascn.resize(na);
    if(na) CUDA_TRY(c,cudaMemcpy(ascn.data(),c->active_scene,sizeof(int)*na,cudaMemcpyDeviceToHost));
    for(int s:scn) if(s==scene) out->n_valid++;
    for(int s:ascn) if(s==scene) out->n_active_blocks++;
    const CGState& g=c->h_cg[scene];
    out->n_interior=g.n_interior;out->cg_iterations=g.iters;out->cg_converged=g.converged;
    out->cg_residual=g.residual;out->cg_tolerance=g.tol;
    const unsigned long long trips=c->h_ctr->total_trips;
    if(trips>c->loop_iters_seen){c->launches+=(long long)(trips-c->loop_iters_seen)*c->graph_kernels_body;c->loop_iters_seen=trips;}
    out->gpu_launches=c->launches;
    return MPM_OK;
}

mpm_status mpm_flag_counts(mpm_context* c,int scene,long long out3[3])
{
    if(bad_scene(c,scene)||!out3||!c->initialized) return MPM_BAD_ARG;
    // The Dirichlet box is that of the particles at the last grid build. The current
    // particle buffer holds the positions after that substep's G2P, so this call reports
    // the box of the current positions, i.e. the one the next substep will build.
    return dispatch(c,[&](auto p)->mpm_status{
        using P=decltype(p);using T=TT<P>;
        DevState<T> S=make_state<P>(c,c->cur,0.0);
        unsigned long long* tmp=nullptr;CUDA_TRY(c,cudaMalloc(&tmp,8*8));
        std::vector<unsigned long long> init(8,0ull);for(int a=0;a<3;++a) init[a]=~0ull;
        CUDA_TRY(c,cudaMemcpy(tmp,init.data(),64,cudaMemcpyHostToDevice));
        k_bbox<T><<<grid_for(c,4),256,0,c->stream>>>(S,scene,tmp,tmp+3);c->launches++;
        std::vector<unsigned long long> h(8);
        CUDA_TRY(c,cudaMemcpyAsync(h.data(),tmp,64,cudaMemcpyDeviceToHost,c->stream));
        CUDA_TRY(c,cudaStreamSynchronize(c->stream));
        auto unord=[](unsigned long long u){long long b=(long long)((u&0x8000000000000000ull)?u^0x8000000000000000ull:~u);double d;std::memcpy(&d,&b,8);return d;};
        const mpm_scene_desc& d=c->scenes[scene].desc;
        int lo[3],hi[3];long long dir=1;
        for(int a=0;a<3;++a){
            T mn=(T)std::max(0.0,unord(h[a])),mx=(T)std::min(1.0,unord(h[3+a]));
            mn=std::max((T)0.,mn);mx=std::min((T)1.,mx);
            auto clampc=[&](T x){int cc=(int)std::floor((double)(x*(T)d.counts[a]));return std::min(std::max(cc,0),d.counts[a]-1);};
            lo[a]=clampc(mn);hi[a]=clampc(mx);dir*=(long long)(hi[a]-lo[a]+1);}
        CUDA_TRY(c,cudaMemsetAsync(tmp+6,0,8,c->stream));
        k_count_in_box<T><<<grid_for(c,4),256,0,c->stream>>>(S,scene,lo[0],lo[1],lo[2],hi[0],hi[1],hi[2],tmp+6);c->launches++;
        unsigned long long both=0;
        CUDA_TRY(c,cudaMemcpyAsync(&both,tmp+6,8,cudaMemcpyDeviceToHost,c->stream));
        CUDA_TRY(c,cudaMemcpyAsync(c->h_cg,c->cg,sizeof(CGState)*c->scenes.size(),cudaMemcpyDeviceToHost,c->stream));
        CUDA_TRY(c,cudaStreamSynchronize(c->stream));
        cudaFree(tmp);
        out3[0]=dir;out3[1]=c->h_cg[scene].n_interior;out3[2]=(long long)both;
        return MPM_OK;});
}

mpm_status mpm_get_interior_nodes(mpm_context* c,int scene,long long capacity,int* coords,double* mass,double* v,double* vstar,long long* n)
{
    if(bad_scene(c,scene)||!n||!c->initialized) return MPM_BAD_ARG;
    return dispatch(c,[&](auto p)->mpm_status{
        using P=decltype(p);using T=TT<P>;
        DevState<T> S=make_state<P>(c,c->cur,0.0);
        unsigned long long* cnt=nullptr;CUDA_TRY(c,cudaMalloc(&cnt,8));
        CUDA_TRY(c,cudaMemsetAsync(cnt,0,8,c->stream));
        const long long cap=std::max<long long>(capacity,0);
        int* dc=nullptr;double *dm=nullptr,*dv=nullptr,*dvs=nullptr;
        if(cap>0){CUDA_TRY(c,cudaMalloc(&dc,sizeof(int)*3*cap));CUDA_TRY(c,cudaMalloc(&dm,8*cap));CUDA_TRY(c,cudaMalloc(&dv,24*cap));CUDA_TRY(c,cudaMalloc(&dvs,24*cap));}
        k_interior_export<T><<<grid_for(c,4),256,0,c->stream>>>(S,scene,cap,dc,dm,dv,dvs,cnt);c->launches++;
        unsigned long long h=0;
        CUDA_TRY(c,cudaMemcpyAsync(&h,cnt,8,cudaMemcpyDeviceToHost,c->stream));
        CUDA_TRY(c,cudaStreamSynchronize(c->stream));
        const long long k=std::min<long long>((long long)h,cap);
        if(k>0){
            if(coords) CUDA_TRY(c,cudaMemcpy(coords,dc,sizeof(int)*3*k,cudaMemcpyDeviceToHost));
            if(mass) CUDA_TRY(c,cudaMemcpy(mass,dm,8*k,cudaMemcpyDeviceToHost));
            if(v) CUDA_TRY(c,cudaMemcpy(v,dv,24*k,cudaMemcpyDeviceToHost));
            if(vstar) CUDA_TRY(c,cudaMemcpy(vstar,dvs,24*k,cudaMemcpyDeviceToHost));}
        cudaFree(cnt);if(dc){cudaFree(dc);cudaFree(dm);cudaFree(dv);cudaFree(dvs);}
        *n=(long long)h;
        return MPM_OK;});
}

mpm_status mpm_get_active_blocks(mpm_context* c,int scene,long long capacity,int* coords,long long* n)
{
    if(bad_scene(c,scene)||!n||!c->initialized) return MPM_BAD_ARG;
    CUDA_TRY(c,cudaMemcpyAsync(c->h_ctr,c->ctr,sizeof(Counters),cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    const long long na=std::min<long long>(c->h_ctr->n_active,c->block_cap);
    std::vector<int> gb(na),sc(na);
    if(na){CUDA_TRY(c,cudaMemcpy(gb.data(),c->active_gb,sizeof(int)*na,cudaMemcpyDeviceToHost));
           CUDA_TRY(c,cudaMemcpy(sc.data(),c->active_scene,sizeof(int)*na,cudaMemcpyDeviceToHost));}
    const HostScene& hs=c->scenes[scene];
    long long k=0;
    for(long long i=0;i<na;++i){
        if(sc[i]!=scene) continue;
        if(coords&&k<capacity){long long lb=gb[i]-hs.block_base;
            coords[3*k]=(int)(lb%hs.nb[0])-1;lb/=hs.nb[0];coords[3*k+1]=(int)(lb%hs.nb[1])-1;coords[3*k+2]=(int)(lb/hs.nb[1])-1;}
        k++;}
    *n=k;
    return MPM_OK;
}

mpm_status mpm_get_sort(mpm_context* c,long long capacity,uint32_t* keys,int* order,int* scene_of,long long* n)
{
    if(!c||!n||!c->initialized) return MPM_BAD_ARG;
    const long long nt=c->n_total;*n=nt;
    if(capacity<nt) return MPM_OK;
    const int fin=c->sort_passes&1;
    std::vector<int> pid(nt),scn(nt);
    if(keys) CUDA_TRY(c,cudaMemcpyAsync(keys,c->keys[fin],sizeof(unsigned)*nt,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(pid.data(),c->pid[c->cur],sizeof(int)*nt,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(scn.data(),c->scn[c->cur],sizeof(int)*nt,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    for(long long i=0;i<nt;++i){
        const int s=scn[i]>=0?scn[i]:-scn[i]-1;
        const long long base=c->scenes[s].pid_ranges.empty()?0:c->scenes[s].pid_ranges[0].first;
        if(order) order[i]=(int)(pid[i]-base);
        if(scene_of) scene_of[i]=s;}
    return MPM_OK;
}

mpm_status mpm_synchronize(mpm_context* c)
{
    if(!c) return MPM_BAD_ARG;
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    return MPM_OK;
}
void* mpm_stream(mpm_context* c){return c?(void*)c->stream:nullptr;}

mpm_status mpm_set_timing(mpm_context* c,int enabled)
{
    if(!c) return MPM_BAD_ARG;
    c->timing=enabled!=0;
    if(c->timing){for(int i=0;i<PH_COUNT;++i){c->phase_ms[i]=0;c->phase_launches[i]=0;}}
    return MPM_OK;
}
int mpm_get_phase_times(mpm_context* c,int capacity,const char** names,double* ms,long long* launches)
{
    if(!c) return 0;
    for(int i=0;i<PH_COUNT&&i<capacity;++i){
        if(names) names[i]=kPhaseNames[i];
        if(ms) ms[i]=c->phase_ms[i];
        if(launches) launches[i]=c->phase_launches[i];}
    return PH_COUNT;
}
mpm_status mpm_time_steps(mpm_context* c,int k,double dt,double* ms)
{
    if(!c||!ms||k<0) return MPM_BAD_ARG;
    cudaEvent_t a,b;
    CUDA_TRY(c,cudaEventCreate(&a));CUDA_TRY(c,cudaEventCreate(&b));
    CUDA_TRY(c,cudaEventRecord(a,c->stream));
    mpm_status s=dispatch(c,[&](auto p){
        using P=decltype(p);
        if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
        CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),c->stream));
        for(int i=0;i<k;++i){mpm_status r=(c->cfg.use_graphs&&!c->timing)?substep_graph<P>(c,dt):substep_eager<P>(c,dt,0);if(r!=MPM_OK) return r;}
        return MPM_OK;});
    if(s!=MPM_OK){cudaEventDestroy(a);cudaEventDestroy(b);return s;}
    CUDA_TRY(c,cudaEventRecord(b,c->stream));
    CUDA_TRY(c,cudaEventSynchronize(b));
    float f=0;cudaEventElapsedTime(&f,a,b);*ms=f;
    cudaEventDestroy(a);cudaEventDestroy(b);
    return collect_status(c);
}

mpm_status mpm_get_cg_iterations(mpm_context* c,int capacity,int* iterations,long long* interior_nodes,int* n_scenes)
{
    if(!c||capacity<0||(capacity>0&&!iterations&&!interior_nodes)) return MPM_BAD_ARG;
    const int ns=(int)c->scenes.size();
    if(n_scenes) *n_scenes=ns;
    if(!c->initialized||capacity==0) return MPM_OK;
    CUDA_TRY(c,cudaMemcpyAsync(c->h_cg,c->cg,sizeof(CGState)*ns,cudaMemcpyDeviceToHost,c->stream));
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    for(int i=0;i<ns&&i<capacity;++i){
        if(iterations) iterations[i]=c->h_cg[i].iters;
        if(interior_nodes) interior_nodes[i]=c->h_cg[i].n_interior;}
    return MPM_OK;
}

mpm_status mpm_selftest_lookback_wait(mpm_context* c,int spin_limit)
{
    if(!c) return MPM_BAD_ARG;
    if(spin_limit<1||spin_limit>OS_SPIN_LIMIT) return fail(c,MPM_BAD_ARG,"spin_limit must be in [1, 2^22]");
    if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
    // two status words in the sort scratch (rewritten by every substep's binning)
    CUDA_TRY(c,cudaMemsetAsync(c->sortws,0,2*sizeof(unsigned),c->stream));
    CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),c->stream));
    k_lookback_selftest<<<1,32,0,c->stream>>>(c->sortws,&c->ctr->error,spin_limit);c->launches++;
    CUDA_TRY(c,cudaGetLastError());
    return collect_status(c);
}


} // extern "C"

// ---------- launch configuration and autotuner ----------
namespace {

mpm_launch_config current_launch(const mpm_context* c)
{
    mpm_launch_config L;
    L.chunk=c->cfg.chunk;L.ctas_hessian=c->minb_hess;L.ctas_p2g=c->minb_p2g;L.ctas_g2p=c->minb_g2p;L.grid_per_sm=c->xfer_grid;
    L.node_grid_per_sm=c->node_grid;
    L.hessian_warp_items=c->hess_warp;
    L.incremental_sort=c->sort_incremental;
    return L;
}
bool is_variant(int v){for(int x:kXferVariants) if(x==v) return true;return false;}
bool same_launch(const mpm_launch_config& a,const mpm_launch_config& b)
{
    return a.chunk==b.chunk&&a.ctas_hessian==b.ctas_hessian&&a.ctas_p2g==b.ctas_p2g&&a.ctas_g2p==b.ctas_g2p&&a.grid_per_sm==b.grid_per_sm&&
           a.node_grid_per_sm==b.node_grid_per_sm&&a.hessian_warp_items==b.hessian_warp_items&&a.incremental_sort==b.incremental_sort;
}
// Work-item capacity for a work-item size: every active block can start a work item, plus
// one per `chunk` particles.
long long chunk_capacity(const mpm_context* c,int chunk){return c->block_cap+c->cfg.max_particles/chunk+16;}

mpm_status apply_launch(mpm_context* c,const mpm_launch_config& L)
{
    if(L.chunk<32||L.chunk>4096||!is_variant(L.ctas_hessian)||!is_variant(L.ctas_p2g)||!is_variant(L.ctas_g2p)||
       L.grid_per_sm<1||L.grid_per_sm>64||L.node_grid_per_sm<1||L.node_grid_per_sm>64||
       L.hessian_warp_items<0||L.hessian_warp_items>2||(L.incremental_sort!=0&&L.incremental_sort!=1)) return fail(c,MPM_BAD_ARG,"launch configuration out of range");
    if(c->buffers_ready&&chunk_capacity(c,L.chunk)>c->chunk_cap){
        CUDA_TRY(c,cudaStreamSynchronize(c->stream));
        CUDA_TRY(c,cudaFree(c->chunk_start));c->chunk_start=nullptr;
        const long long cap=chunk_capacity(c,L.chunk);
        CUDA_TRY(c,cudaMalloc((void**)&c->chunk_start,sizeof(int)*cap));
        c->chunk_cap=cap;}
    c->cfg.chunk=L.chunk;c->minb_hess=L.ctas_hessian;c->minb_p2g=L.ctas_p2g;c->minb_g2p=L.ctas_g2p;c->xfer_grid=L.grid_per_sm;
    c->node_grid=L.node_grid_per_sm;c->hess_warp=L.hessian_warp_items;c->sort_incremental=L.incremental_sort;
    c->graph_valid=false;c->frame_graph_valid=false;
    return MPM_OK;
}

// A device copy of the particle state (the current buffer's first n_total slots) and of
// the per-scene solver state.
struct StateSnapshot {
    void* state=nullptr; int* pid=nullptr; int* scn=nullptr; CGState* cg=nullptr;
    int cur=0;
    ~StateSnapshot(){cudaFree(state);cudaFree(pid);cudaFree(scn);cudaFree(cg);}
};
mpm_status snapshot_take(mpm_context* c,StateSnapshot& s)
{
    const long long n=c->n_total,pc=c->cfg.max_particles;const size_t ts=c->tsize;
    CUDA_TRY(c,cudaMalloc(&s.state,ts*NB_FIELDS*std::max<long long>(n,1)));
    CUDA_TRY(c,cudaMalloc((void**)&s.pid,sizeof(int)*std::max<long long>(n,1)));
    CUDA_TRY(c,cudaMalloc((void**)&s.scn,sizeof(int)*std::max<long long>(n,1)));
    CUDA_TRY(c,cudaMalloc((void**)&s.cg,sizeof(CGState)*c->cfg.max_scenes));
    s.cur=c->cur;
    for(int k=0;k<NB_FIELDS;++k)
        CUDA_TRY(c,cudaMemcpyAsync((char*)s.state+ts*k*n,(char*)c->pstate[s.cur]+ts*k*pc,ts*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(s.pid,c->pid[s.cur],sizeof(int)*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(s.scn,c->scn[s.cur],sizeof(int)*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(s.cg,c->cg,sizeof(CGState)*c->cfg.max_scenes,cudaMemcpyDeviceToDevice,c->stream));
    return MPM_OK;
}
mpm_status snapshot_restore(mpm_context* c,const StateSnapshot& s)
{
    const long long n=c->n_total,pc=c->cfg.max_particles;const size_t ts=c->tsize;
    c->cur=s.cur;c->order_epoch++;
    for(int k=0;k<NB_FIELDS;++k)
        CUDA_TRY(c,cudaMemcpyAsync((char*)c->pstate[s.cur]+ts*k*pc,(char*)s.state+ts*k*n,ts*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(c->pid[s.cur],s.pid,sizeof(int)*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(c->scn[s.cur],s.scn,sizeof(int)*n,cudaMemcpyDeviceToDevice,c->stream));
    CUDA_TRY(c,cudaMemcpyAsync(c->cg,s.cg,sizeof(CGState)*c->cfg.max_scenes,cudaMemcpyDeviceToDevice,c->stream));
    return MPM_OK;
}

// One trial: restore the state, one untimed substep, then k substeps timed one by one.
template<class P> mpm_status tune_trial(mpm_context* c,const StateSnapshot& snap,double dt,int k,double* median_ms)
{
    mpm_status s=snapshot_restore(c,snap);if(s!=MPM_OK) return s;
    CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),c->stream));
    auto one=[&]()->mpm_status{return (c->cfg.use_graphs&&!c->timing)?substep_graph<P>(c,dt):substep_eager<P>(c,dt,0);};
    s=one();if(s!=MPM_OK) return s;
    std::vector<cudaEvent_t> ev(k+1);
    for(auto& e:ev) CUDA_TRY(c,cudaEventCreate(&e));
    mpm_status r=MPM_OK;
    CUDA_TRY(c,cudaEventRecord(ev[0],c->stream));
    for(int i=0;i<k&&r==MPM_OK;++i){r=one();if(r==MPM_OK&&cudaEventRecord(ev[i+1],c->stream)!=cudaSuccess) r=MPM_CUDA_ERROR;}
    std::vector<double> ms;
    if(r==MPM_OK&&cudaEventSynchronize(ev[k])==cudaSuccess){
        for(int i=0;i<k;++i){float f=0;cudaEventElapsedTime(&f,ev[i],ev[i+1]);ms.push_back(f);}}
    else if(r==MPM_OK) r=MPM_CUDA_ERROR;
    for(auto& e:ev) cudaEventDestroy(e);
    if(r!=MPM_OK) return r;
    const mpm_status st=collect_status(c);
    if(st!=MPM_OK&&st!=MPM_CG_NOT_CONVERGED) return st;
    std::sort(ms.begin(),ms.end());
    *median_ms=ms[ms.size()/2];
    return MPM_OK;
}

template<class P> mpm_status autotune_impl(mpm_context* c,double dt,int k,mpm_tune_result* out)
{
    if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
    if(!(dt>0.)||k<1||k>1000) return fail(c,MPM_BAD_ARG,"autotune needs dt > 0 and 1..1000 substeps per trial");
    const long long saved_substeps=c->substeps,saved_launches=c->launches;
    long long saved_phase[PH_COUNT];for(int i=0;i<PH_COUNT;++i) saved_phase[i]=c->phase_launches[i];
    StateSnapshot snap;
    mpm_status s=snapshot_take(c,snap);if(s!=MPM_OK) return s;
    const mpm_launch_config initial=current_launch(c);
    mpm_launch_config best=initial;double best_ms=0;int trials=0;
    s=tune_trial<P>(c,snap,dt,k,&best_ms);trials++;
    if(s!=MPM_OK){apply_launch(c,initial);snapshot_restore(c,snap);cudaStreamSynchronize(c->stream);return s;}
    const double initial_ms=best_ms;
    const int chunks[]={256,512,1024,2048};
    const int variants[]={3,4,5,6};
    const int grids[]={4,8,12,16};
    const int node_grids[]={1,2,4,8};
    const int forms[]={HESS_AUTO,HESS_CTA,HESS_WARP};
    const int binnings[]={0,1};
    // coordinate 0: the Hessian's form (chosen per launch, work items per CTA or per warp), then work-item
    // size, the three occupancy variants, transfer grid, node-kernel grid and the binning
    // (full sort or merge into the previous order); a second sweep revisits every
    // coordinate from the first sweep's best (interactions such as work-item size against
    // occupancy), timing only candidates not yet tried
    std::vector<mpm_launch_config> tried{initial};
    for(int sweep=0;sweep<2;++sweep)
    for(int coord=0;coord<8;++coord){
        const int* vals=coord==0?forms:coord==7?binnings:coord==1?chunks:coord==5?grids:coord==6?node_grids:variants;
        const int nvals=coord==0?3:coord==7?2:4;
        for(int i=0;i<nvals;++i){
            mpm_launch_config L=best;
            int* field=coord==0?&L.hessian_warp_items:coord==1?&L.chunk:coord==2?&L.ctas_hessian:coord==3?&L.ctas_p2g:
                       coord==4?&L.ctas_g2p:coord==5?&L.grid_per_sm:coord==6?&L.node_grid_per_sm:&L.incremental_sort;
            *field=vals[i];
            if(same_launch(L,best)) continue;
            bool seen=false;for(const auto& t:tried) seen|=same_launch(L,t);
            if(seen) continue;
            tried.push_back(L);
            if(apply_launch(c,L)!=MPM_OK) continue;
            double ms=0;
            const mpm_status t=tune_trial<P>(c,snap,dt,k,&ms);trials++;
            if(t==MPM_CUDA_ERROR){apply_launch(c,initial);snapshot_restore(c,snap);cudaStreamSynchronize(c->stream);return t;}
            if(t==MPM_OK&&ms<best_ms){best_ms=ms;best=L;}}}
    s=apply_launch(c,best);
    if(s==MPM_OK) s=snapshot_restore(c,snap);
    CUDA_TRY(c,cudaStreamSynchronize(c->stream));
    c->substeps=saved_substeps;c->launches=saved_launches;
    for(int i=0;i<PH_COUNT;++i) c->phase_launches[i]=saved_phase[i];
    if(out){out->chosen=best;out->initial=initial;out->ms_per_substep=best_ms;out->ms_per_substep_initial=initial_ms;out->trials=trials;}
    return s;
}

} // namespace

extern "C" {

mpm_status mpm_get_time(mpm_context* c,double* t)
{
    if(!c||!t) return MPM_BAD_ARG;
    *t=c->time;
    return MPM_OK;
}
mpm_status mpm_set_time(mpm_context* c,double t)
{
    if(!c||!std::isfinite(t)) return MPM_BAD_ARG;
    c->time=t;
    return MPM_OK;
}
mpm_status mpm_advance_to_time(mpm_context* c,double target_time,double cfl,int max_substeps,int* substeps_done)
{
    if(!c) return MPM_BAD_ARG;
    if(substeps_done) *substeps_done=0;
    if(!(cfl>0.)||max_substeps<1||!std::isfinite(target_time)) return fail(c,MPM_BAD_ARG,"advance_to_time needs cfl > 0, max_substeps >= 1 and a finite target");
    if(!c->initialized) return fail(c,MPM_NOT_READY,"mpm_initialize has not run");
    if(!(target_time>c->time)) return MPM_OK;
    return dispatch(c,[&](auto p)->mpm_status{
        using P=decltype(p);
        FrameState& hf=*c->h_frame;
        hf=FrameState{};
        hf.time=c->time;hf.target=target_time;hf.cfl=cfl;hf.dt_min=1e-6;hf.dt_max=5e-3;hf.max_substeps=max_substeps;
        CUDA_TRY(c,cudaMemcpyAsync(c->frame,&hf,sizeof(FrameState),cudaMemcpyHostToDevice,c->stream));
        CUDA_TRY(c,cudaMemsetAsync(&c->ctr->error,0,2*sizeof(unsigned),c->stream));
        c->last_dt=-1;   // dt is now written on the device; a later fixed-dt substep sets it again
        if(c->cfg.use_graphs&&!c->timing){
            if(!c->frame_graph_valid||c->graph_ntotal!=c->n_total){mpm_status s=build_frame_graphs<P>(c);if(s!=MPM_OK) return s;}
            CUDA_TRY(c,cudaGraphLaunch(c->fgexec[c->cur],c->stream));
            CUDA_TRY(c,cudaMemcpyAsync(c->h_frame,c->frame,sizeof(FrameState),cudaMemcpyDeviceToHost,c->stream));
            CUDA_TRY(c,cudaStreamSynchronize(c->stream));
            c->cur^=(c->h_frame->substeps&1);c->order_epoch++;
            c->launches+=(long long)c->h_frame->substeps*c->frame_kernels_per_substep;}
        else{
            for(;;){
                k_cfl<TT<P>><<<grid_for(c,4),NODE_THREADS,0,c->stream>>>(make_state<P>(c,c->cur,0.),c->frame,c->d_dt,0ull,0);c->launches++;
                mpm_status s=substep_eager<P>(c,0.,0,true);if(s!=MPM_OK) return s;
                c->substeps--;   // counted below
                CUDA_TRY(c,cudaMemcpyAsync(c->h_frame,c->frame,sizeof(FrameState),cudaMemcpyDeviceToHost,c->stream));
                CUDA_TRY(c,cudaStreamSynchronize(c->stream));
                if(c->h_frame->done) break;}}
        c->substeps+=c->h_frame->substeps;
        c->time=c->h_frame->time;
        if(substeps_done) *substeps_done=c->h_frame->substeps;
        return collect_status(c);});
}

mpm_status mpm_get_launch_config(mpm_context* c,mpm_launch_config* out)
{
    if(!c||!out) return MPM_BAD_ARG;
    *out=current_launch(c);
    return MPM_OK;
}
mpm_status mpm_set_launch_config(mpm_context* c,const mpm_launch_config* cfg)
{
    if(!c||!cfg) return MPM_BAD_ARG;
    return apply_launch(c,*cfg);
}
mpm_status mpm_autotune(mpm_context* c,double dt,int substeps,mpm_tune_result* out)
{
    if(!c) return MPM_BAD_ARG;
    return dispatch(c,[&](auto p){return autotune_impl<decltype(p)>(c,dt,substeps,out);});
}

} // extern "C"
