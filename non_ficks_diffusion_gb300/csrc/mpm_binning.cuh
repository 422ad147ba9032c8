// mpm_binning.cuh — integer work of the substep: cell keys, a stable LSD radix sort of
// (key, slot) pairs, device-wide exclusive scans, work-item (chunk) compaction and node-
// block activation. Replaces the reference's per-substep grid rebuild and particle
// binning (Compute_Bounding_Box / Rasterize_Voxels / Group_Particles,
// MPM_Example.cpp:236-311, 464-485). All results are deterministic and bit-exact.
#pragma once
#include "mpm_device.cuh"

namespace mpm {

constexpr int RS_THREADS=256, RS_WARPS=RS_THREADS/32;
// Keys per thread of a radix tile: small inputs use short tiles so that every SM has one.
constexpr int RS_ITEMS_SMALL=4, RS_ITEMS=16, RS_TILE=RS_THREADS*RS_ITEMS;
constexpr long long RS_SMALL_N=1<<21;
__host__ __device__ constexpr int rs_items(long long n){return n<RS_SMALL_N?RS_ITEMS_SMALL:RS_ITEMS;}
// Tile size of the one-sweep passes: short tiles give small inputs one per SM; long ones
// keep the look-back chain short on large inputs.
__host__ __device__ constexpr int os_items(long long n){return n<(1LL<<18)?RS_ITEMS_SMALL:RS_ITEMS;}
constexpr int SC_THREADS=512, SC_ITEMS=8, SC_SEG=SC_THREADS*SC_ITEMS;

__device__ __forceinline__ unsigned lanemask_lt(){unsigned m;asm("mov.u32 %0, %%lanemask_lt;":"=r"(m));return m;}

// ---- cell keys (key layout documented at mpm_get_sort) ----
template<class T> __device__ __forceinline__ T mul_rn(T a,T b);
template<> __device__ __forceinline__ float mul_rn<float>(float a,float b){return __fmul_rn(a,b);}
template<> __device__ __forceinline__ double mul_rn<double>(double a,double b){return __dmul_rn(a,b);}

// Cell key of particle slot i of the current buffer, scene s >= 0, position x. A
// non-finite position or one outside the grid removes the particle (its scene id becomes
// -(s+1)), sets an error flag and gives KEY_SENTINEL.
template<class T> __device__ __forceinline__ unsigned cell_key(const DevState<T>& S,long long i,int s,const T (&x)[3])
{
    const SceneDev<T>& sc=S.scenes[s];
    int c[3];bool ok=true,fin=true;
#pragma unroll
    for(int a=0;a<3;++a){
        if(!isfinite(x[a])) fin=false;
        const T f=floor(mul_rn<T>(x[a],sc.inv_dx[a]));
        c[a]=fin&&f>T(-8)&&f<T(sc.counts[a]+8)?(int)f:-100;
        if(c[a]<-3||c[a]>sc.counts[a]+1) ok=false;}
    if(!fin){atomicOr(&S.ctr->error,ERR_NONFINITE);atomicMax(&S.ctr->bad_scene1,(unsigned)s+1u);}
    else if(!ok) atomicOr(&S.ctr->error,ERR_OUT_OF_GRID);
    if(!(fin&&ok)){S.scn_cur[i]=-(s+1);return KEY_SENTINEL;}
    const int b0=(c[0]+4)>>2,b1=(c[1]+4)>>2,b2=(c[2]+4)>>2;
    const int l=((c[0]+4)&3)|(((c[1]+4)&3)<<2)|(((c[2]+4)&3)<<4);
    const long long gb=sc.block_base+b0+(long long)sc.nb[0]*(b1+(long long)sc.nb[1]*b2);
    return (unsigned)((gb<<6)|l);
}
// Cell keys of the slots i0 + 32j + lane (j < N; KEY_SENTINEL at and above n and for
// removed particles). Every load of the batch is issued before any key is formed, so a
// warp waits for memory once per batch instead of once per slot.
template<class T,int N> __device__ __forceinline__ void particle_keys(const DevState<T>& S,long long i0,int lane,long long n,unsigned (&key)[N])
{
    int sj[N];T x[N][3];
#pragma unroll
    for(int j=0;j<N;++j){
        const long long i=i0+j*32+lane;
        const bool in=i<n;
        sj[j]=in?S.scn_cur[i]:-1;
#pragma unroll
        for(int a=0;a<3;++a) x[j][a]=in?S.pcur[(long long)(FX+a)*S.pcap+i]:T(0);}
#pragma unroll
    for(int j=0;j<N;++j) key[j]=sj[j]<0?KEY_SENTINEL:cell_key(S,i0+j*32+lane,sj[j],x[j]);
}

// Adds the warp's digits d of the lanes with `in` to the shared histogram h: one atomic
// when all 32 agree, one per lane when at most four lanes take part, else one per distinct
// digit (the lowest lane of each group adds the group's count; match.any is the slow
// path).
__device__ __forceinline__ void count_digit(unsigned* h,unsigned d,bool in,int lane)
{
    const unsigned d0=__shfl_sync(0xffffffffu,d,0);
    if(__all_sync(0xffffffffu,in&&d==d0)){if(lane==0) atomicAdd(&h[d0],32u);return;}
    if(__popc(__ballot_sync(0xffffffffu,in))<=4){if(in) atomicAdd(&h[d],1u);return;}
    const unsigned peers=__match_any_sync(0xffffffffu,in?d:256u+lane);
    if(in&&(peers&lanemask_lt())==0u) atomicAdd(&h[d],(unsigned)__popc(peers));
}
// Keys and identity values of all slots (one warp per 32*KEY_ITEMS consecutive slots).
// Also counts the 8-bit digits of the sorted block bits (shifts 6, 14, 22, 30) for the
// first `passes` (<= 4) sort passes into hist[pass][256] (zeroed beforehand), so that every
// one-sweep pass knows its digit offsets without a separate histogram pass.
constexpr int KEY_ITEMS=8;
template<class T> __global__ void __launch_bounds__(256) k_keys(DevState<T> S,unsigned* keys,int* vals,unsigned* hist,int passes)
{
    pdl_enter();
    __shared__ unsigned h[4][256];
    for(int t=threadIdx.x;t<4*256;t+=blockDim.x) (&h[0][0])[t]=0;
    __syncthreads();
    unsigned nv=0;
    const int lane=threadIdx.x&31;
    const long long n=S.n_total;
    const long long wstride=(long long)gridDim.x*(blockDim.x>>5)*(32*KEY_ITEMS);
    for(long long i0=((long long)blockIdx.x*(blockDim.x>>5)+(threadIdx.x>>5))*(32*KEY_ITEMS);i0<n;i0+=wstride){
        unsigned key[KEY_ITEMS];
        particle_keys<T,KEY_ITEMS>(S,i0,lane,n,key);
#pragma unroll
        for(int j=0;j<KEY_ITEMS;++j){
            const long long i=i0+j*32+lane;
            const bool in=i<n;
            if(key[j]!=KEY_SENTINEL) nv++;
            if(in){keys[i]=key[j];vals[i]=(int)i;}
            // particles arrive sorted by block, so a warp's digits mostly agree
            for(int p=0;p<passes;++p) count_digit(h[p],(key[j]>>(6+8*p))&255u,in,lane);}
    }
    // one atomic per warp
    for(int o=16;o>0;o>>=1) nv+=__shfl_xor_sync(0xffffffffu,nv,o);
    if((threadIdx.x&31)==0&&nv) atomicAdd(&S.ctr->n_valid,nv);
    __syncthreads();
    for(int t=threadIdx.x;t<passes*256;t+=blockDim.x){const unsigned v=(&h[0][0])[t];if(v) atomicAdd(&hist[t],v);}
}

// ---- one-sweep radix pass (decoupled look-back) ----
// One kernel per 8-bit pass. Tiles are taken in the order of an atomic counter, so every
// tile before the one a CTA holds is held by a CTA that has already started. A tile ranks
// its keys stably (as k_radix_scatter), publishes its per-digit counts, then walks back
// over the earlier tiles' published words until it meets an inclusive prefix; the sum is
// the tile's offset inside each digit. Status word per (tile, digit): 2 flag bits
// (0 none, 1 count of the tile, 2 inclusive prefix) over a 30-bit count; the array and
// the tile counter start at zero. A wait that exceeds its spin limit sets ERR_SORT_WAIT.
constexpr unsigned OS_AGG=1u<<30, OS_PRE=2u<<30, OS_MASK=(1u<<30)-1u;
constexpr int OS_SPIN_LIMIT=1<<22;
constexpr int OS_LOOKBACK=4;
__device__ __forceinline__ unsigned os_load(const unsigned* p){return *(const volatile unsigned*)p;}
// Waits (bounded: at most spin_limit polls) until *p is published; returns it, or 0 after
// setting ERR_SORT_WAIT.
__device__ __forceinline__ unsigned os_wait(const unsigned* p,unsigned* error,int spin_limit=OS_SPIN_LIMIT)
{
    unsigned v=os_load(p);int spins=0;
    while((v&~OS_MASK)==0u&&++spins<spin_limit){__nanosleep(32);v=os_load(p);}
    if((v&~OS_MASK)==0u) atomicOr(error,ERR_SORT_WAIT);
    return v;
}
template<int ITEMS> __global__ void __launch_bounds__(RS_THREADS) k_onesweep(const unsigned* __restrict__ kin,const int* __restrict__ vin,
                                                  unsigned* __restrict__ kout,int* __restrict__ vout,long long n,int shift,
                                                  const unsigned* __restrict__ hist,unsigned* status,unsigned* tile_counter,
                                                  int num_tiles,unsigned* error,const unsigned* n_dev=nullptr)
{
    pdl_enter();
    if(n_dev){n=*n_dev;num_tiles=(int)((n+RS_THREADS*ITEMS-1)/(RS_THREADS*ITEMS));}   // count known on the device only
    __shared__ unsigned wcnt[RS_WARPS][256];
    __shared__ unsigned base_digit[256],tile_off[256];
    __shared__ int tile_sh;
    const int w=threadIdx.x>>5,lane=threadIdx.x&31;
    {   // exclusive scan of the pass's digit histogram: where each digit starts
        const unsigned v=hist[threadIdx.x];
        unsigned incl=v;
#pragma unroll
        for(int o=1;o<32;o<<=1){const unsigned u=__shfl_up_sync(0xffffffffu,incl,o);if(lane>=o) incl+=u;}
        if(lane==31) wcnt[0][w]=incl;
        __syncthreads();
        unsigned wbase=0;
        for(int ww=0;ww<w;++ww) wbase+=wcnt[0][ww];
        base_digit[threadIdx.x]=wbase+incl-v;
        __syncthreads();}
    for(;;){
        if(threadIdx.x==0) tile_sh=(int)atomicAdd(tile_counter,1u);
        __syncthreads();
        const int tile=tile_sh;
        if(tile>=num_tiles) break;                     // uniform
        for(int t=threadIdx.x;t<RS_WARPS*256;t+=RS_THREADS) (&wcnt[0][0])[t]=0;
        __syncthreads();
        const long long base=(long long)tile*RS_THREADS*ITEMS+(long long)w*(ITEMS*32);
        unsigned k[ITEMS];unsigned short r[ITEMS];
#pragma unroll
        for(int j=0;j<ITEMS;++j){
            const long long idx=base+j*32+lane;
            const bool valid=idx<n;
            k[j]=valid?kin[idx]:0u;
            const unsigned d=(k[j]>>shift)&255u;
            const unsigned peers=__match_any_sync(0xffffffffu,valid?d:(256u+lane));
            const unsigned rank=__popc(peers&lanemask_lt());
            const unsigned before=valid?wcnt[w][d]:0u;
            __syncwarp();
            if(valid&&rank==0) wcnt[w][d]=before+__popc(peers);
            __syncwarp();
            r[j]=(unsigned short)(before+rank);}
        __syncthreads();
        {   // one digit per thread: offsets of the warps, the tile's count, look-back
            const int d=threadIdx.x;unsigned run=0;
#pragma unroll
            for(int ww=0;ww<RS_WARPS;++ww){const unsigned c=wcnt[ww][d];wcnt[ww][d]=run;run+=c;}
            unsigned* my=status+(long long)tile*256+d;
            if(tile==0) atomicExch(my,OS_PRE|run);
            else{
                atomicExch(my,OS_AGG|run);
                // walk back OS_LOOKBACK tiles per round trip: the loads are independent, and
                // the frontier of inclusive prefixes advances by one window per trip
                unsigned excl=0;bool done=false;
                for(int t=tile-1;t>=0&&!done;t-=OS_LOOKBACK){
                    unsigned v[OS_LOOKBACK];
#pragma unroll
                    for(int u=0;u<OS_LOOKBACK;++u) v[u]=t-u>=0?os_load(status+(long long)(t-u)*256+d):OS_PRE;
#pragma unroll
                    for(int u=0;u<OS_LOOKBACK;++u){
                        if(done||t-u<0) break;
                        unsigned x=v[u];
                        if((x&~OS_MASK)==0u){x=os_wait(status+(long long)(t-u)*256+d,error);if((x&~OS_MASK)==0u){done=true;break;}}
                        excl+=x&OS_MASK;
                        if((x&~OS_MASK)==OS_PRE) done=true;}}
                atomicExch(my,OS_PRE|(excl+run));
                run=excl;}
            tile_off[d]=base_digit[d]+(tile==0?0u:run);}
        __syncthreads();
#pragma unroll
        for(int j=0;j<ITEMS;++j){
            const long long idx=base+j*32+lane;
            if(idx<n){
                const unsigned d=(k[j]>>shift)&255u;
                const long long pos=(long long)tile_off[d]+wcnt[w][d]+r[j];
                kout[pos]=k[j];vout[pos]=vin?vin[idx]:(int)idx;}}
        __syncthreads();
    }
}

// Non-template kernels here are static: every translation unit that includes this header
// gets its own copy.
// ---- radix sort: 8-bit digits, per-tile histograms laid out [digit][tile] ----
template<int ITEMS> static __global__ void __launch_bounds__(RS_THREADS) k_radix_hist(const unsigned* __restrict__ keys,long long n,int shift,
                                                           unsigned* __restrict__ counts,int num_tiles)
{
    __shared__ unsigned h[256];
    for(int tile=blockIdx.x;tile<num_tiles;tile+=gridDim.x){
        h[threadIdx.x]=0;
        __syncthreads();
        const long long base=(long long)tile*RS_THREADS*ITEMS;
#pragma unroll 4
        for(int j=0;j<ITEMS;++j){
            const long long idx=base+j*RS_THREADS+threadIdx.x;
            if(idx<n) atomicAdd(&h[(keys[idx]>>shift)&255u],1u);}
        __syncthreads();
        counts[(long long)threadIdx.x*num_tiles+tile]=h[threadIdx.x];
        __syncthreads();
    }
}

// Stable scatter: warp w of a tile owns the contiguous keys [w*32*ITEMS, (w+1)*32*ITEMS) and walks
// them 32 at a time in index order; peers with the same digit are ranked by lane order
// (match.any) on top of the warp's running per-digit count; warps are then offset by an
// exclusive scan over warps per digit.
template<int ITEMS> static __global__ void __launch_bounds__(RS_THREADS) k_radix_scatter(const unsigned* __restrict__ kin,const int* __restrict__ vin,
                                                              unsigned* __restrict__ kout,int* __restrict__ vout,long long n,int shift,
                                                              const unsigned* __restrict__ offsets,int num_tiles)
{
    __shared__ unsigned wcnt[RS_WARPS][256];
    const int w=threadIdx.x>>5,lane=threadIdx.x&31;
    for(int tile=blockIdx.x;tile<num_tiles;tile+=gridDim.x){
        for(int t=threadIdx.x;t<RS_WARPS*256;t+=RS_THREADS) (&wcnt[0][0])[t]=0;
        __syncthreads();
        const long long base=(long long)tile*RS_THREADS*ITEMS+(long long)w*(ITEMS*32);
        unsigned k[ITEMS];unsigned short r[ITEMS];
#pragma unroll
        for(int j=0;j<ITEMS;++j){
            const long long idx=base+j*32+lane;
            const bool valid=idx<n;
            k[j]=valid?kin[idx]:0u;
            const unsigned d=(k[j]>>shift)&255u;
            const unsigned peers=__match_any_sync(0xffffffffu,valid?d:(256u+lane));
            const unsigned rank=__popc(peers&lanemask_lt());
            const unsigned before=valid?wcnt[w][d]:0u;
            __syncwarp();
            if(valid&&rank==0) wcnt[w][d]=before+__popc(peers);
            __syncwarp();
            r[j]=(unsigned short)(before+rank);}
        __syncthreads();
        {   // exclusive scan over warps, one digit per thread
            const int d=threadIdx.x;unsigned run=0;
#pragma unroll
            for(int ww=0;ww<RS_WARPS;++ww){const unsigned c=wcnt[ww][d];wcnt[ww][d]=run;run+=c;}}
        __syncthreads();
#pragma unroll
        for(int j=0;j<ITEMS;++j){
            const long long idx=base+j*32+lane;
            if(idx<n){
                const unsigned d=(k[j]>>shift)&255u;
                const long long pos=(long long)offsets[(long long)d*num_tiles+tile]+wcnt[w][d]+r[j];
                kout[pos]=k[j];vout[pos]=vin?vin[idx]:(int)idx;}}
        __syncthreads();
    }
}

// ---- device-wide exclusive scan of uint32 (segments of SC_SEG, three kernels) ----
template<class F> __device__ __forceinline__ unsigned seg_sum(F get,long long n,long long seg)
{
    unsigned s=0;const long long base=seg*SC_SEG;
#pragma unroll
    for(int j=0;j<SC_ITEMS;++j){const long long i=base+j*SC_THREADS+threadIdx.x;if(i<n) s+=get(i);}
    __shared__ unsigned red[SC_THREADS/32];
    for(int o=16;o>0;o>>=1) s+=__shfl_xor_sync(0xffffffffu,s,o);
    if((threadIdx.x&31)==0) red[threadIdx.x>>5]=s;
    __syncthreads();
    unsigned t=0;
    if(threadIdx.x<32){t=threadIdx.x<SC_THREADS/32?red[threadIdx.x]:0u;for(int o=16;o>0;o>>=1) t+=__shfl_xor_sync(0xffffffffu,t,o);}
    __syncthreads();
    return t;   // valid in thread 0
}
// CTA-wide exclusive scan of one value per thread; returns the prefix, *total the sum.
__device__ __forceinline__ unsigned cta_exclusive_scan(unsigned v,unsigned* total)
{
    __shared__ unsigned wsum[32];
    const int lane=threadIdx.x&31,w=threadIdx.x>>5,nw=(blockDim.x+31)>>5;
    unsigned x=v;
#pragma unroll
    for(int o=1;o<32;o<<=1){const unsigned y=__shfl_up_sync(0xffffffffu,x,o);if(lane>=o) x+=y;}
    if(lane==31) wsum[w]=x;
    __syncthreads();
    if(w==0){unsigned s=lane<nw?wsum[lane]:0u;
#pragma unroll
        for(int o=1;o<32;o<<=1){const unsigned y=__shfl_up_sync(0xffffffffu,s,o);if(lane>=o) s+=y;}
        wsum[lane]=s;}
    __syncthreads();
    const unsigned excl=x-v+(w>0?wsum[w-1]:0u);
    if(total) *total=wsum[nw-1];
    __syncthreads();
    return excl;
}

static __global__ void __launch_bounds__(SC_THREADS) k_scan_sums(const unsigned* __restrict__ in,long long n,unsigned* __restrict__ sums)
{
    const long long nseg=(n+SC_SEG-1)/SC_SEG;
    for(long long seg=blockIdx.x;seg<nseg;seg+=gridDim.x){
        const unsigned t=seg_sum([&](long long i){return in[i];},n,seg);
        if(threadIdx.x==0) sums[seg]=t;}
}
// One CTA: exclusive scan of sums[0..nseg) in place; writes the grand total to *total and,
// if cap_check>=0, flags ERR_CAPACITY when the total exceeds it.
static __global__ void __launch_bounds__(1024) k_scan_top(unsigned* sums,long long nseg,unsigned* total,long long cap_check,unsigned* err)
{
    unsigned carry=0;
    for(long long base=0;base<nseg;base+=blockDim.x){
        const long long i=base+threadIdx.x;
        const unsigned v=i<nseg?sums[i]:0u;
        unsigned tot;const unsigned e=cta_exclusive_scan(v,&tot);
        if(i<nseg) sums[i]=carry+e;
        carry+=tot;}
    if(threadIdx.x==0){
        if(total) *total=carry;
        if(cap_check>=0&&(long long)carry>cap_check&&err) atomicOr(err,ERR_CAPACITY);}
}
static __global__ void __launch_bounds__(SC_THREADS) k_scan_apply(const unsigned* __restrict__ in,unsigned* __restrict__ out,long long n,
                                                           const unsigned* __restrict__ sums)
{
    const long long nseg=(n+SC_SEG-1)/SC_SEG;
    for(long long seg=blockIdx.x;seg<nseg;seg+=gridDim.x){
        const long long base=seg*SC_SEG+(long long)threadIdx.x*SC_ITEMS;
        unsigned v[SC_ITEMS],s=0;
#pragma unroll
        for(int j=0;j<SC_ITEMS;++j){v[j]=base+j<n?in[base+j]:0u;s+=v[j];}
        const unsigned off=sums[seg]+cta_exclusive_scan(s,nullptr);
        unsigned run=off;
#pragma unroll
        for(int j=0;j<SC_ITEMS;++j){if(base+j<n) out[base+j]=run;run+=v[j];}
    }
}

// Exclusive prefix of the CTA's segment total `total` over segments taken in the order of
// an atomic counter (decoupled look-back, one word per segment, zeroed beforehand; see
// k_onesweep for the flags). Called by every thread; warp 0 publishes the segment's
// aggregate, sums earlier aggregates back to the nearest inclusive prefix and publishes
// its own. The frontier of inclusive prefixes advances by one look-back window per memory
// round trip, so warp 0 reads CP_LOADS words per lane (CP_LOADS*32 segments per trip).
constexpr int CP_LOADS=1;
__device__ __forceinline__ unsigned chained_prefix(unsigned* status,long long seg,unsigned total,unsigned* err,
                                                   int spin_limit=OS_SPIN_LIMIT)
{
    __shared__ unsigned pre;
    if(threadIdx.x<32){
        const int lane=threadIdx.x;
        unsigned excl=0;
        if(seg==0){if(lane==0) atomicExch(status,OS_PRE|total);}
        else{
            if(lane==0) atomicExch(status+seg,OS_AGG|total);
            for(long long t=seg-1;t>=0;t-=32*CP_LOADS){
                // lane l reads segments t-l*CP_LOADS-u, nearest first; below 0 reads as a
                // zero prefix
                unsigned v[CP_LOADS];
#pragma unroll
                for(int u=0;u<CP_LOADS;++u){const long long q=t-(long long)lane*CP_LOADS-u;v[u]=q>=0?os_load(status+q):OS_PRE;}
                int fp=CP_LOADS;                        // the lane's nearest prefix (or failed wait)
#pragma unroll
                for(int u=CP_LOADS-1;u>=0;--u){
                    if((v[u]&~OS_MASK)==0u) v[u]=os_wait(status+(t-(long long)lane*CP_LOADS-u),err,spin_limit);
                    if((v[u]&~OS_MASK)==OS_PRE||(v[u]&~OS_MASK)==0u) fp=u;}
                const unsigned isp=__ballot_sync(0xffffffffu,fp<CP_LOADS);
                const int stop=isp?__ffs(isp)-1:32;     // nearest lane with a prefix
                unsigned c=0;
#pragma unroll
                for(int u=0;u<CP_LOADS;++u) if(lane<stop||(lane==stop&&u<=fp)) c+=v[u]&OS_MASK;
#pragma unroll
                for(int o=16;o>0;o>>=1) c+=__shfl_xor_sync(0xffffffffu,c,o);
                excl+=c;
                if(isp) break;}
            if(lane==0) atomicExch(status+seg,OS_PRE|(excl+total));}
        if(lane==0) pre=excl;}
    __syncthreads();
    const unsigned r=pre;
    __syncthreads();
    return r;
}
__device__ __forceinline__ long long next_segment(unsigned* counter)
{
    __shared__ long long seg;
    if(threadIdx.x==0) seg=(long long)atomicAdd(counter,1u);
    __syncthreads();
    const long long r=seg;
    __syncthreads();
    return r;
}
// ---- incremental binning: exact stable order from the previous substep's ----
// The particle slots arrive ordered by their previous block p(i) (the previous sort's
// keys, which P2G rewrote in slot order), so p is non-decreasing. A slot is "moved" when
// its new block b(i) differs from p(i); the unmoved slots are then already sorted by
// (b, i), and moved_before(x) counts the moved slots below x, nm(x) = x - moved_before(x)
// the unmoved ones. A moved slot q with new block b goes after exactly
// R = nm(anchor) unmoved slots, anchor = the first slot whose previous block is >= b when
// b > p(q) (all such slots lie above q), the first whose previous block is > b when
// b < p(q) (all below q). With the moved slots sorted stably by b (j-th in (b, q) order),
//   moved j  -> j + R_j      unmoved slot i -> nm(i) + #{j : R_j <= nm(i)}
// which are the positions of a stable sort by b, for any non-decreasing p: stale or
// constant previous keys cost speed (more moved slots), never exactness. Blocks are
// compared as the sort passes see them: (key >> 6) & umask.
constexpr int MV_THREADS=256, MV_ITEMS=8;
__device__ __forceinline__ unsigned key_block(unsigned key,unsigned umask){return (key>>6)&umask;}
__device__ __forceinline__ long long moved_before(const uint2* __restrict__ words,long long x,long long n,long long m)
{
    if(x>=n) return m;
    const uint2 wd=words[x>>5];
    return (long long)wd.x+__popc(wd.y&((1u<<(x&31))-1u));
}
// Keys of all slots into knew and the moved mask of every 32 slots into words[].y (one
// warp per 32*MV_ITEMS consecutive slots), and the digit histograms of the moved keys for
// the first `passes` sort passes.
template<class T> __global__ void __launch_bounds__(MV_THREADS) k_keys_moved(DevState<T> S,const unsigned* __restrict__ prev,
        unsigned* __restrict__ knew,uint2* __restrict__ words,unsigned* hist,int passes,unsigned umask)
{
    pdl_enter();
    __shared__ unsigned h[4][256];
    for(int t=threadIdx.x;t<4*256;t+=blockDim.x) (&h[0][0])[t]=0;
    __syncthreads();
    const int lane=threadIdx.x&31;
    const long long n=S.n_total;
    const long long wstride=(long long)gridDim.x*(blockDim.x>>5)*(32*MV_ITEMS);
    unsigned nv=0;
    for(long long base=((long long)blockIdx.x*(blockDim.x>>5)+(threadIdx.x>>5))*(32*MV_ITEMS);base<n;base+=wstride){
        unsigned key[MV_ITEMS],pk[MV_ITEMS];
#pragma unroll
        for(int j=0;j<MV_ITEMS;++j){const long long i=base+j*32+lane;pk[j]=i<n?prev[i]:0u;}
        particle_keys<T,MV_ITEMS>(S,base,lane,n,key);
#pragma unroll
        for(int j=0;j<MV_ITEMS;++j){
            const long long i=base+j*32+lane;
            const bool in=i<n;
            const unsigned k=key[j];
            if(k!=KEY_SENTINEL) nv++;
            const bool moved=in&&key_block(k,umask)!=key_block(pk[j],umask);
            if(in) knew[i]=k;
            const unsigned mv=__ballot_sync(0xffffffffu,moved);
            if(lane==0&&base+j*32<n) words[(base+j*32)>>5].y=mv;
            if(mv) for(int p=0;p<passes;++p) count_digit(h[p],(k>>(6+8*p))&255u,moved,lane);}
    }
    for(int o=16;o>0;o>>=1) nv+=__shfl_xor_sync(0xffffffffu,nv,o);
    if(lane==0&&nv) atomicAdd(&S.ctr->n_valid,nv);
    __syncthreads();
    for(int t=threadIdx.x;t<passes*256;t+=blockDim.x){const unsigned v=(&h[0][0])[t];if(v) atomicAdd(&hist[t],v);}
}
// Anchor of moved slot q with new block u and previous block pu != u: a galloping search
// over the previous keys from q outward (most moves go to a neighbouring block, whose
// slots are close).
__device__ __forceinline__ long long moved_anchor(const unsigned* __restrict__ prev,long long n,long long q,unsigned u,unsigned pu,unsigned umask)
{
    long long lo,hi;
    if(u>pu){           // first slot above q whose previous block is >= u
        lo=q+1;long long step=1;
        for(;;){const long long x=q+step;
            if(x>=n){hi=n;break;}
            if(key_block(prev[x],umask)>=u){hi=x;break;}
            lo=x+1;step<<=1;}
        while(lo<hi){const long long mid=(lo+hi)>>1;if(key_block(prev[mid],umask)<u) lo=mid+1; else hi=mid;}}
    else{               // first slot (at most q) whose previous block is > u
        hi=q;long long step=1;
        for(;;){const long long x=q-step;
            if(x<0){lo=0;break;}
            if(key_block(prev[x],umask)<=u){lo=x+1;break;}
            hi=x;step<<=1;}
        while(lo<hi){const long long mid=(lo+hi)>>1;if(key_block(prev[mid],umask)<=u) lo=mid+1; else hi=mid;}}
    return lo;
}
// Compaction of the moved slots in slot order, MC_WORDS words (32 slots each) per tile,
// tiles in ticket order with a decoupled look-back over their moved counts (own status
// words, zeroed beforehand). words[].x becomes the moved count before each 32 slots. Each
// thread writes the slots of its words' moved bits; then the warp's lanes take the warp's
// entries round-robin for the key and the anchor search, so that a dense word does not
// serialise its searches on one thread. The last tile stores the moved count in *m_total.
constexpr int MC_THREADS=256, MC_WPT=2, MC_WORDS=MC_THREADS*MC_WPT, MC_TILE=MC_WORDS*32;
static __global__ void __launch_bounds__(MC_THREADS) k_moved_compact(const unsigned* __restrict__ prev,const unsigned* __restrict__ knew,
        uint2* __restrict__ words,long long n,unsigned umask,unsigned* status,unsigned* tile_counter,unsigned* err,
        unsigned* __restrict__ mkey,int* __restrict__ mslot,int* __restrict__ manchor,unsigned* m_total)
{
    pdl_enter();
    __shared__ unsigned wtot[MC_THREADS/32];
    const int lane=threadIdx.x&31,w=threadIdx.x>>5;
    const long long nwords=(n+31)>>5,num_tiles=(nwords+MC_WORDS-1)/MC_WORDS;
    for(;;){
        const long long tile=next_segment(tile_counter);
        if(tile>=num_tiles) break;                        // uniform
        const long long wb=tile*MC_WORDS+(long long)threadIdx.x*MC_WPT;
        unsigned mw[MC_WPT];unsigned c=0;
#pragma unroll
        for(int h=0;h<MC_WPT;++h){mw[h]=wb+h<nwords?words[wb+h].y:0u;c+=__popc(mw[h]);}
        unsigned x=c;                                      // inclusive warp scan, then across warps
#pragma unroll
        for(int o=1;o<32;o<<=1){const unsigned y=__shfl_up_sync(0xffffffffu,x,o);if(lane>=o) x+=y;}
        if(lane==31) wtot[w]=x;
        __syncthreads();
        unsigned wex=0,tot=0;
#pragma unroll
        for(int ww=0;ww<MC_THREADS/32;++ww){const unsigned t=wtot[ww];if(ww<w) wex+=t;tot+=t;}
        const unsigned toff=chained_prefix(status,tile,tot,err);
        unsigned pos=toff+wex+x-c;
        const unsigned wfirst=toff+wex,wend=toff+wex+__shfl_sync(0xffffffffu,x,31);
#pragma unroll
        for(int h=0;h<MC_WPT;++h){
            if(wb+h<nwords) words[wb+h].x=pos;
            unsigned mm=mw[h];
            while(mm){const int b=__ffs(mm)-1;mm&=mm-1;mslot[pos++]=(int)((wb+h)*32+b);}}
        __syncwarp();
        for(unsigned p=wfirst+lane;p<wend;p+=32){
            const long long q=mslot[p];
            const unsigned key=knew[q];
            mkey[p]=key;
            manchor[p]=(int)moved_anchor(prev,n,q,key_block(key,umask),key_block(prev[q],umask),umask);}
        if(tile==num_tiles-1&&threadIdx.x==0) *m_total=toff+tot;
    }
}
// Moved slots to their final positions (j-th of the sorted list: sorted key skey[j], its
// compaction index sc[j]): R = nm(anchor) unmoved slots precede it. Their R in sorted
// order into rs.
static __global__ void __launch_bounds__(256) k_moved_out(const unsigned* __restrict__ skey,const int* __restrict__ sc,
        const int* __restrict__ mslot,const int* __restrict__ manchor,const uint2* __restrict__ words,
        const unsigned* __restrict__ m_total,long long n,unsigned* __restrict__ kout,int* __restrict__ vout,int* __restrict__ rs)
{
    pdl_enter();
    const long long m=*m_total;
    for(long long j=blockIdx.x*(long long)blockDim.x+threadIdx.x;j<m;j+=(long long)gridDim.x*blockDim.x){
        const int c=sc[j];
        const long long a=manchor[c];
        const long long r=a-moved_before(words,a,n,m);
        const long long d=j+r;
        kout[d]=skey[j];vout[d]=mslot[c];rs[j]=(int)r;}
}
// Unmoved slots to their final positions, MU_TILE slots per tile, tiles blockIdx.x +
// k*gridDim.x. A tile's unmoved ranks lie in [nm(t0), nm(t1)), so the moved entries ranked
// among them form one range [lower_bound(rs, nm(t0)), lower_bound(rs, nm(t1))) of rs. The
// bounds of up to MU_ROUND of a CTA's tiles are searched at once, one per thread, before
// those tiles are streamed. A short range (the usual case) goes through registers 32
// entries at a time, each slot counting the entries <= its rank by a 6-step shuffle
// search; a long one by a binary search per slot.
constexpr int MU_THREADS=256, MU_ITEMS=8, MU_TILE=MU_THREADS*MU_ITEMS, MU_ROUND=MU_THREADS/2, MU_SHORT=256;
__device__ __forceinline__ long long rank_lower_bound(const int* __restrict__ rs,long long lo,long long hi,long long x)
{
    while(lo<hi){const long long mid=(lo+hi)>>1;if((long long)rs[mid]<x) lo=mid+1; else hi=mid;}
    return lo;
}
// #{lanes l : v_l <= r} for values v sorted across the lanes
__device__ __forceinline__ int warp_count_le(int v,int r)
{
    int pos=0;
#pragma unroll
    for(int st=16;st>0;st>>=1) if(__shfl_sync(0xffffffffu,v,pos+st-1)<=r) pos+=st;
    if(__shfl_sync(0xffffffffu,v,pos)<=r) pos++;
    return pos;
}
static __global__ void __launch_bounds__(MU_THREADS) k_merge_unmoved(const unsigned* __restrict__ knew,const uint2* __restrict__ words,
        const int* __restrict__ rs,const unsigned* __restrict__ m_total,long long n,unsigned* __restrict__ kout,int* __restrict__ vout)
{
    pdl_enter();
    __shared__ long long jb[MU_ROUND][2];
    const long long m=*m_total;
    const int lane=threadIdx.x&31;
    const long long num_tiles=(n+MU_TILE-1)/MU_TILE;
    const long long my_tiles=blockIdx.x<num_tiles?(num_tiles-1-blockIdx.x)/gridDim.x+1:0;
    for(long long k0=0;k0<my_tiles;k0+=MU_ROUND){
        {   const long long k=k0+(threadIdx.x>>1);
            if(k<my_tiles){
                const long long t0=(blockIdx.x+k*gridDim.x)*MU_TILE;
                const long long x=(threadIdx.x&1)?(t0+MU_TILE<n?t0+MU_TILE:n):t0;
                jb[threadIdx.x>>1][threadIdx.x&1]=rank_lower_bound(rs,0,m,x-moved_before(words,x,n,m));}}
        __syncthreads();
        const long long kend=k0+MU_ROUND<my_tiles?k0+MU_ROUND:my_tiles;
        for(long long k=k0;k<kend;++k){
            const long long t0=(blockIdx.x+k*gridDim.x)*MU_TILE,t1=t0+MU_TILE<n?t0+MU_TILE:n;
            const long long jlo=jb[k-k0][0],jhi=jb[k-k0][1];
            uint2 wd[MU_ITEMS];unsigned kn[MU_ITEMS];
#pragma unroll
            for(int q=0;q<MU_ITEMS;++q){
                const long long i=t0+q*MU_THREADS+threadIdx.x;
                wd[q]=i<t1?words[i>>5]:make_uint2(0u,0xffffffffu);
                kn[q]=i<t1?knew[i]:0u;}
            int r[MU_ITEMS];long long a[MU_ITEMS];
#pragma unroll
            for(int q=0;q<MU_ITEMS;++q){
                const long long i=t0+q*MU_THREADS+threadIdx.x;
                r[q]=(int)(i-(long long)(wd[q].x+__popc(wd[q].y&lanemask_lt())));a[q]=jlo;}
            if(jhi-jlo<=MU_SHORT){                         // uniform
                for(long long c=jlo;c<jhi;c+=32){
                    const int v=c+lane<jhi?rs[c+lane]:0x7fffffff;
#pragma unroll
                    for(int q=0;q<MU_ITEMS;++q) a[q]+=warp_count_le(v,r[q]);}}
            else{
#pragma unroll
                for(int q=0;q<MU_ITEMS;++q) a[q]=rank_lower_bound(rs,jlo,jhi,(long long)r[q]+1);}
#pragma unroll
            for(int q=0;q<MU_ITEMS;++q){
                const long long i=t0+q*MU_THREADS+threadIdx.x;
                if(i<t1&&!((wd[q].y>>lane)&1u)){kout[r[q]+a[q]]=kn[q];vout[r[q]+a[q]]=(int)i;}}}
        __syncthreads();
    }
}

// CTA-wide exclusive max-scan of one value per thread (identity `lo`).
__device__ __forceinline__ long long cta_exclusive_max(long long v,long long lo,long long* total=nullptr)
{
    __shared__ long long wmax[32];
    const int lane=threadIdx.x&31,w=threadIdx.x>>5,nw=(blockDim.x+31)>>5;
    long long x=v;
#pragma unroll
    for(int o=1;o<32;o<<=1){const long long y=__shfl_up_sync(0xffffffffu,x,o);if(lane>=o&&y>x) x=y;}
    if(lane==31) wmax[w]=x;
    __syncthreads();
    if(w==0){long long s=lane<nw?wmax[lane]:lo;
#pragma unroll
        for(int o=1;o<32;o<<=1){const long long y=__shfl_up_sync(0xffffffffu,s,o);if(lane>=o&&y>s) s=y;}
        wmax[lane]=s;}
    __syncthreads();
    long long prev=__shfl_up_sync(0xffffffffu,x,1);
    if(lane==0) prev=lo;
    const long long wprev=w>0?wmax[w-1]:lo;
    const long long r=prev>wprev?prev:wprev;
    if(total) *total=wmax[nw-1];
    __syncthreads();
    return r;
}
// Work-item heads and block activation in one pass over the sorted keys, CH_SEG keys per
// segment, segments taken in ticket order.
// Work items: each particle's block start is the last block head at or before it. Heads
// inside the segment come from a CTA max-scan; the start of the block the segment begins
// in comes from a look-back over the earlier segments' published last heads (each
// segment publishes its own before it looks back, so the walk ends at the nearest one
// that has a head). Work-item counts then go through the chained prefix. The last
// segment stores the number of work items and flags ERR_CAPACITY beyond the capacity.
// Activation: a particle with local cell coordinate l on an axis reaches the neighbour
// block below when l==0 and above when l==3 (stencil offsets -1..1), so it needs the
// product of those offset ranges over the three axes: a 27-bit mask, bit
// (ox+1)+3(oy+1)+9(oz+1). The segment's particles are numbered by block run, the masks
// are OR-ed per run in shared memory, and each run's needed blocks are set in the bitmap
// once. The active set is exactly the blocks that some particle's stencil touches.
constexpr int CH_THREADS=256, CH_ITEMS=8, CH_SEG=CH_THREADS*CH_ITEMS;
template<class T> __global__ void __launch_bounds__(CH_THREADS) k_chunk_heads(DevState<T> S,long long n,int chunk,unsigned* status,
                                                                               unsigned* head_status,unsigned* counter)
{
    pdl_enter();
    static_assert(CH_SEG<65536,"work-item and run counts share one scan word");
    __shared__ unsigned run_block[CH_SEG],run_mask[CH_SEG];
    __shared__ long long sbase[MAX_SCENES];
    __shared__ int snb[MAX_SCENES][2];
    __shared__ long long seg_start;
    const unsigned* __restrict__ keys=S.keys;
    Counters* ctr=S.ctr;
    const long long cap=S.chunk_cap;
    const unsigned nv=ctr->n_valid;
    const long long nseg=(n+CH_SEG-1)/CH_SEG;
    const int lane=threadIdx.x&31;
    for(int k=threadIdx.x;k<S.n_scenes;k+=CH_THREADS){
        sbase[k]=S.scene_block_base[k];snb[k][0]=S.scenes[k].nb[0];snb[k][1]=S.scenes[k].nb[1];}
    for(;;){
        const long long seg=next_segment(counter);  // its barrier also publishes the scene table
        if(seg>=nseg) break;
        const long long i0=seg*CH_SEG;
        const long long base=i0+(long long)threadIdx.x*CH_ITEMS;
        unsigned kk[CH_ITEMS+1],cl[CH_ITEMS];
#pragma unroll
        for(int j=0;j<=CH_ITEMS;++j){
            const long long i=base+j-1;
            const bool in=i>=0&&i<(long long)nv;
            const unsigned k=in?keys[i]:0u;
            kk[j]=in?(k>>6):0xffffffffu;
            if(j>0) cl[j-1]=k&63u;}
        long long last=-1;
        unsigned hr=0;                                 // run starts after the segment's first particle
#pragma unroll
        for(int j=0;j<CH_ITEMS;++j){
            const long long i=base+j;
            if(i<(long long)nv&&(i==0||kk[j]!=kk[j+1])){last=i;if(i>i0) hr++;}}
        long long seg_last;
        const long long carry=cta_exclusive_max(last,-1,&seg_last);
        if(threadIdx.x<32){
            // publish this segment's last head (value 0: none), then find the start of the
            // block that holds the segment's first particle
            if(lane==0) atomicExch(head_status+seg,OS_PRE|(seg_last>=0?(unsigned)(seg_last-i0)+1u:0u));
            long long bs=i0;
            const bool first_is_head=i0==0||i0>=(long long)nv||__shfl_sync(0xffffffffu,kk[0]!=kk[1],0);
            if(!first_is_head){
                for(long long t=seg-1;t>=0;t-=32){
                    const long long q=t-lane;
                    unsigned v=q>=0?os_load(head_status+q):OS_PRE;
                    if((v&~OS_MASK)==0u) v=os_wait(head_status+q,&ctr->error);
                    const bool failed=(v&~OS_MASK)==0u;
                    const unsigned hit=__ballot_sync(0xffffffffu,failed||(v&OS_MASK)!=0u);
                    if(hit){
                        const int src=__ffs(hit)-1;
                        const unsigned vs=__shfl_sync(0xffffffffu,v,src);
                        bs=(vs&~OS_MASK)==0u?i0:(t-src)*CH_SEG+(long long)(vs&OS_MASK)-1;
                        break;}}}
            if(lane==0) seg_start=bs;}
        __syncthreads();
        long long bs=carry>=0?carry:seg_start;
        unsigned f=0,s=0;
#pragma unroll
        for(int j=0;j<CH_ITEMS;++j){
            const long long i=base+j;
            if(i>=(long long)nv) break;
            if(i==0||kk[j]!=kk[j+1]) bs=i;
            const unsigned b=((i-bs)%chunk)==0?1u:0u;f|=b<<j;s+=b;}
        unsigned tot;
        const unsigned local=cta_exclusive_scan(s|(hr<<16),&tot);
        const unsigned ntot=tot&0xffffu;
        const unsigned nruns=i0<(long long)nv?(tot>>16)+1u:0u;
        // each run's first particle writes the run's block id and clears its mask
        const unsigned r0=local>>16;
        {unsigned r=r0;
#pragma unroll
        for(int j=0;j<CH_ITEMS;++j){
            const long long i=base+j;
            if(i>=(long long)nv) break;
            const bool head=i==0||kk[j]!=kk[j+1];
            if(head&&i>i0) r++;
            if(head||i==i0){run_block[r]=kk[j+1];run_mask[r]=0u;}}}
        const unsigned pre=chained_prefix(status,seg,ntot,&ctr->error);
        // stencil masks: OR-ed in registers over the thread's consecutive particles (runs
        // that end inside the thread go to shared memory directly), then the part of the
        // thread's first run by a segmented OR-scan over the lanes (lanes with the same first
        // run are consecutive) and the part of its last run by the thread
        {unsigned rc=r0,mc=0u,mfirst=0u;bool first_open=true;
#pragma unroll
        for(int j=0;j<CH_ITEMS;++j){
            const long long i=base+j;
            if(i>=(long long)nv) break;
            if(i>i0&&kk[j]!=kk[j+1]){
                if(first_open){mfirst=mc;first_open=false;}
                else if(mc) atomicOr(&run_mask[rc],mc);
                rc++;mc=0u;}
            const unsigned l=cl[j];
            const unsigned lx=l&3u,ly=(l>>2)&3u,lz=l>>4;
            // offset ranges per axis (bit 0: -1, bit 1: 0, bit 2: +1), spread into 3x3x3
            const unsigned rx=2u|(lx==0u?1u:0u)|(lx==3u?4u:0u);
            const unsigned ry=2u|(ly==0u?1u:0u)|(ly==3u?4u:0u);
            const unsigned rz=2u|(lz==0u?1u:0u)|(lz==3u?4u:0u);
            const unsigned mxy=rx*((ry&1u)|((ry&2u)<<2)|((ry&4u)<<4));
            mc|=mxy*((rz&1u)|((rz&2u)<<8)|((rz&4u)<<16));}
        if(first_open){mfirst=mc;mc=0u;}
        unsigned x=mfirst;
#pragma unroll
        for(int o=1;o<32;o<<=1){
            const unsigned y=__shfl_down_sync(0xffffffffu,x,o),ky=__shfl_down_sync(0xffffffffu,r0,o);
            if(lane+o<32&&ky==r0) x|=y;}
        const unsigned kp=__shfl_up_sync(0xffffffffu,r0,1);
        if(x&&(lane==0||kp!=r0)) atomicOr(&run_mask[r0],x);
        if(mc) atomicOr(&run_mask[rc],mc);}
        __syncthreads();
        for(unsigned t=threadIdx.x;t<nruns*27u;t+=CH_THREADS){
            const unsigned r=t/27u,o=t-r*27u;
            if(((run_mask[r]>>o)&1u)==0u) continue;
            const int ox=(int)(o%3u)-1,oy=(int)((o/3u)%3u)-1,oz=(int)(o/9u)-1;
            const long long gb=(long long)run_block[r];
            const int sc=scene_of_block(sbase,S.n_scenes,gb);
            const long long g2=gb+ox+(long long)snb[sc][0]*(oy+(long long)snb[sc][1]*oz);
            atomicOr(&S.bitmap[g2>>5],1u<<(g2&31));}
        unsigned pos=pre+(local&0xffffu);
#pragma unroll
        for(int j=0;j<CH_ITEMS;++j) if((f>>j)&1u){if(pos<cap) S.chunk_start[pos]=(int)(base+j);pos++;}
        if(seg==nseg-1&&threadIdx.x==0){
            ctr->n_chunks=pre+ntot;
            if((long long)(pre+ntot)>cap) atomicOr(&ctr->error,ERR_CAPACITY);}
    }
}

// Active-block indices in one pass: popcounts, chained prefix, assignment in global block
// order, one bitmap word per thread (segments of SC_THREADS words, so small grids still
// spread over several CTAs) and one lane per set bit. The last segment stores the number
// of active blocks and flags ERR_CAPACITY.
constexpr int BM_SEG=SC_THREADS;
template<class T> __global__ void __launch_bounds__(SC_THREADS) k_bitmap_index(DevState<T> S,unsigned* status,unsigned* counter)
{
    pdl_enter();
    __shared__ unsigned wbits[BM_SEG],wpre[BM_SEG];    // the segment's words and their first index
    const long long words=S.bitmap_words;
    const long long nseg=(words+BM_SEG-1)/BM_SEG;
    const int lane=threadIdx.x&31,warp=threadIdx.x>>5,nw=SC_THREADS/32;
    for(;;){
        const long long seg=next_segment(counter);
        if(seg>=nseg) break;
        const long long wi=seg*BM_SEG+threadIdx.x;
        const unsigned wv=wi<words?S.bitmap[wi]:0u;
        unsigned tot;
        const unsigned local=cta_exclusive_scan((unsigned)__popc(wv),&tot);
        const unsigned pre=chained_prefix(status,seg,tot,&S.ctr->error);
        wbits[threadIdx.x]=wv;wpre[threadIdx.x]=pre+local;
        __syncthreads();
        for(int w=warp;w<BM_SEG;w+=nw){
            const unsigned m=wbits[w];
            if(m==0u) continue;                        // uniform over the warp
            if((m>>lane)&1u){
                const unsigned idx=wpre[w]+__popc(m&lanemask_lt());
                const long long gb=(seg*BM_SEG+w)*32+lane;
                if(idx<S.block_cap){
                    S.blockmap[gb]=(int)idx;S.active_gb[idx]=(int)gb;
                    S.active_scene[idx]=scene_of_block(S.scene_block_base,S.n_scenes,gb);}
                else S.blockmap[gb]=-1;}}   // beyond the capacity: no node storage (ERR_CAPACITY below)
        if(seg==nseg-1&&threadIdx.x==0){
            S.ctr->n_active=pre+tot;
            if((long long)(pre+tot)>S.block_cap) atomicOr(&S.ctr->error,ERR_CAPACITY);}
        __syncthreads();
    }
}

} // namespace mpm
