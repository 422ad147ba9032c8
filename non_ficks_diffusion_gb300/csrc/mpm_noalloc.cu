// mpm_noalloc.cu — the stable radix sort of (cell key, index) pairs, callable without any
// device allocation.
//
// Some callers cannot allocate device memory at the point where they sort: a host that
// records its frame loop into a CUDA graph (cudaMalloc is not allowed while a stream is
// being captured), a real-time loop that must not take cudaMalloc's implicit device
// synchronisation, or an embedding framework that owns all device memory through its own
// allocator. They pass their key and value arrays in device memory; the sort's working
// memory (ping-pong buffers, per-tile digit histograms, scan partial sums) comes from the
// fixed static device array below, reserved when the library is loaded on a GPU and held
// until the process exits.
#include "mpm_gb300.h"
#include "mpm_binning.cuh"

#include <cuda.h>   // CUcontext and CUresult only: the two driver functions are looked up through the runtime

#include <algorithm>
#include <mutex>

using namespace mpm;

namespace {

constexpr long long kMaxPairs=MPM_NOALLOC_SORT_MAX;
constexpr long long kMaxTiles=(kMaxPairs+RS_TILE-1)/RS_TILE;
constexpr long long kCounts=256*kMaxTiles;
constexpr long long kSums=(kCounts+SC_SEG-1)/SC_SEG+16;

// One static scratch area per device: ping-pong keys and values, digit counts, scan sums.
struct NoallocScratch {
    unsigned keys[kMaxPairs];
    int vals[kMaxPairs];
    unsigned counts[kCounts];
    unsigned sums[kSums];
};
static __device__ __align__(256) NoallocScratch g_noalloc_scratch;

// Device address of the scratch. In host code the symbol itself is only a host-side
// stand-in; its device address comes from cudaGetSymbolAddress with the device current.
// That address belongs to the module loaded in the current context, so it is cached per
// device together with the identity of the context it was looked up in (cuCtxGetId: unique
// for the life of the process). A context created anew on the device (after
// cudaDeviceReset, or the primary context released and retained again) gets a new identity
// and the address is looked up again.
typedef CUresult (*FnCtxGetCurrent)(CUcontext*);
typedef CUresult (*FnCtxGetId)(CUcontext,unsigned long long*);
struct CachedScratch { unsigned long long ctx_id; NoallocScratch* ptr; };

std::mutex g_mutex;
CachedScratch g_cache[64]={};
FnCtxGetCurrent g_ctx_get_current=nullptr;
FnCtxGetId g_ctx_get_id=nullptr;

// Identity of the calling thread's current context; 0 when none is current.
bool current_context_id(unsigned long long* id)
{
    if(!g_ctx_get_current||!g_ctx_get_id){
        void* f1=nullptr;void* f2=nullptr;cudaDriverEntryPointQueryResult q1,q2;
        if(cudaGetDriverEntryPointByVersion("cuCtxGetCurrent",&f1,12000,cudaEnableDefault,&q1)!=cudaSuccess||
           cudaGetDriverEntryPointByVersion("cuCtxGetId",&f2,12000,cudaEnableDefault,&q2)!=cudaSuccess||
           q1!=cudaDriverEntryPointSuccess||q2!=cudaDriverEntryPointSuccess||!f1||!f2) return false;
        g_ctx_get_current=(FnCtxGetCurrent)f1;g_ctx_get_id=(FnCtxGetId)f2;}
    CUcontext ctx=nullptr;
    if(g_ctx_get_current(&ctx)!=CUDA_SUCCESS) return false;
    *id=0;
    if(!ctx) return true;
    return g_ctx_get_id(ctx,id)==CUDA_SUCCESS;
}

NoallocScratch* scratch_for(int dev)
{
    std::lock_guard<std::mutex> lock(g_mutex);
    if(dev<0||dev>=64) return nullptr;
    unsigned long long id=0;
    if(!current_context_id(&id)) return nullptr;
    if(id!=0&&g_cache[dev].ptr&&g_cache[dev].ctx_id==id) return g_cache[dev].ptr;
    void* p=nullptr;
    if(cudaGetSymbolAddress(&p,g_noalloc_scratch)!=cudaSuccess) return nullptr;   // makes the device's context current
    if(!current_context_id(&id)||id==0) return nullptr;
    g_cache[dev].ctx_id=id;g_cache[dev].ptr=(NoallocScratch*)p;
    return g_cache[dev].ptr;
}

// Launches one kernel and returns that launch's own status (an error left behind by
// earlier, unrelated work in the process is neither reported nor cleared here).
template<class... KA,class... A> cudaError_t launch(void(*k)(KA...),int grid,int block,cudaStream_t st,A&&... a)
{
    cudaLaunchConfig_t cfg={};
    cfg.gridDim=dim3((unsigned)grid);cfg.blockDim=dim3((unsigned)block);cfg.dynamicSmemBytes=0;cfg.stream=st;
    return cudaLaunchKernelEx(&cfg,k,std::forward<A>(a)...);
}

} // namespace

extern "C" mpm_status mpm_sort_pairs_noalloc(const uint32_t* keys_in,const int32_t* vals_in,uint32_t* keys_out,int32_t* vals_out,
                                             long long n,int begin_bit,int end_bit,void* stream)
{
    if(n<0||n>kMaxPairs||!keys_out||!vals_out||(n>0&&!keys_in)) return MPM_BAD_ARG;
    if(begin_bit<0||end_bit>32||begin_bit>=end_bit) return MPM_BAD_ARG;
    if((const void*)keys_in==(const void*)keys_out||(vals_in&&(const void*)vals_in==(const void*)vals_out)) return MPM_BAD_ARG;
    if(n==0) return MPM_OK;
    int dev=0;
    if(cudaGetDevice(&dev)!=cudaSuccess) return MPM_CUDA_ERROR;
    NoallocScratch* sc=scratch_for(dev);
    if(!sc) return MPM_CUDA_ERROR;
    cudaStream_t st=(cudaStream_t)stream;
    int num_sms=0;
    if(cudaDeviceGetAttribute(&num_sms,cudaDevAttrMultiProcessorCount,dev)!=cudaSuccess) return MPM_CUDA_ERROR;
    const int passes=(end_bit-begin_bit+7)/8;
    const int num_tiles=(int)((n+RS_TILE-1)/RS_TILE);
    const int g=std::max(1,std::min(num_tiles,4*num_sms));
    const long long m=256LL*num_tiles,nseg=(m+SC_SEG-1)/SC_SEG;
    const int gs=(int)std::max<long long>(1,std::min<long long>(nseg,8LL*num_sms));
    // Pass p writes to the caller's output when (passes-1-p) is even, so the last pass
    // always lands there; the other passes use the static ping-pong buffers.
    const unsigned* kin=keys_in;const int* vin=vals_in;
    for(int p=0;p<passes;++p){
        const bool to_out=((passes-1-p)%2)==0;
        unsigned* kout=to_out?keys_out:sc->keys;int* vout=to_out?vals_out:sc->vals;
        const int shift=begin_bit+8*p;
        cudaError_t e=launch(k_radix_hist<RS_ITEMS>,g,RS_THREADS,st,kin,n,shift,sc->counts,num_tiles);
        if(e==cudaSuccess) e=launch(k_scan_sums,gs,SC_THREADS,st,(const unsigned*)sc->counts,m,sc->sums);
        if(e==cudaSuccess) e=launch(k_scan_top,1,1024,st,sc->sums,nseg,(unsigned*)nullptr,-1LL,(unsigned*)nullptr);
        if(e==cudaSuccess) e=launch(k_scan_apply,gs,SC_THREADS,st,(const unsigned*)sc->counts,sc->counts,m,(const unsigned*)sc->sums);
        if(e==cudaSuccess) e=launch(k_radix_scatter<RS_ITEMS>,g,RS_THREADS,st,kin,vin,kout,vout,n,shift,(const unsigned*)sc->counts,num_tiles);
        if(e!=cudaSuccess) return MPM_CUDA_ERROR;
        kin=kout;vin=vout;}
    return MPM_OK;
}
