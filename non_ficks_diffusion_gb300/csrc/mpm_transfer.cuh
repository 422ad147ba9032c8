// mpm_transfer.cuh — particle<->grid transfers, grid update and the implicit CG of one
// substep, as sm_103a kernels over the block-sparse grid of mpm_device.cuh.
//
// Work items ("chunks") are runs of at most `chunk` sorted particles inside one 4x4x4
// block. A chunk's stencils cover the 6x6x6 nodes from one below to one above its block,
// so every transfer kernel stages that tile in shared memory: P2G-type kernels accumulate
// into per-warp copies of it and flush them with one global vector atomic per touched
// node; G2P-type kernels load it once and gather from it. P2G writes each chunk's
// particles in cell order, and threads take them with a stride of chunk/32, so lanes of a
// warp sit in different cells and rarely scatter to the same nodes.
#pragma once
#include "mpm_device.cuh"

namespace mpm {

constexpr int TILE=6, TILE_N=TILE*TILE*TILE;
// Shared-memory layout of a 6x6x6 node tile: node (x, y, z) at x + TSY y + TSZ z, TILE_S
// words per channel. The z stride of 40 (not 36) spreads the cells of a block over the 32
// banks so that, with the cell order below, a warp's 32 scatter or gather addresses
// mostly fall in distinct banks.
constexpr int TSY=6, TSZ=40, TILE_S=5+5*TSY+5*TSZ+1;
__host__ __device__ constexpr int tile_addr(int tx,int ty,int tz){return tx+TSY*ty+TSZ*tz;}
__host__ __device__ constexpr int tile_addr(int t){return tile_addr(t%TILE,(t/TILE)%TILE,t/(TILE*TILE));}
constexpr int XFER_THREADS=128;   // CTA size of the transfer kernels = particles per work item
constexpr int NODE_THREADS=256;

// ---------- helpers ----------
__device__ __forceinline__ float tfma(float a,float b,float c){return fmaf(a,b,c);}
__device__ __forceinline__ double tfma(double a,double b,double c){return fma(a,b,c);}
// Packed pairs of single-precision operations: one instruction does the work of two, and
// each half rounds exactly like the scalar fmaf / multiply.
__device__ __forceinline__ float2 pfma(float2 a,float2 b,float2 c){return __ffma2_rn(a,b,c);}
__device__ __forceinline__ float2 pmul(float2 a,float2 b){return __fmul2_rn(a,b);}
__device__ __forceinline__ float2 pdup(float a){return make_float2(a,a);}
__device__ __forceinline__ float tpow(float a,float b){return powf(a,b);}
__device__ __forceinline__ double tpow(double a,double b){return pow(a,b);}
__device__ __forceinline__ unsigned lane_bits_below(){unsigned m;asm("mov.u32 %0, %%lanemask_lt;":"=r"(m));return m;}
template<class T> __device__ __forceinline__ T sub_rn(T a,T b);
template<> __device__ __forceinline__ float sub_rn<float>(float a,float b){return __fsub_rn(a,b);}
template<> __device__ __forceinline__ double sub_rn<double>(double a,double b){return __dsub_rn(a,b);}
template<class T> __device__ __forceinline__ T add_rn(T a,T b);
template<> __device__ __forceinline__ float add_rn<float>(float a,float b){return __fadd_rn(a,b);}
template<> __device__ __forceinline__ double add_rn<double>(double a,double b){return __dadd_rn(a,b);}
template<class T> __device__ __forceinline__ T fmul_rn(T a,T b);
template<> __device__ __forceinline__ float fmul_rn<float>(float a,float b){return __fmul_rn(a,b);}
template<> __device__ __forceinline__ double fmul_rn<double>(double a,double b){return __dmul_rn(a,b);}

__device__ __forceinline__ void atomic_add_v3(V4<float>* p,float x,float y,float z,float w)
{atomicAdd(reinterpret_cast<float4*>(p),make_float4(x,y,z,w));}
__device__ __forceinline__ void atomic_add_v3(V4<double>* p,double x,double y,double z,double w)
{atomicAdd(&p->x,x);atomicAdd(&p->y,y);atomicAdd(&p->z,z);if(w!=0.) atomicAdd(&p->w,w);}

// Chunk geometry: particle range, block, scene and the 27 neighbour active indices.
template<class T> struct ChunkInfo {
    int s,e,scene;
    int b[3];        // block coordinates inside the scene
    long long gb;
};
// The geometry of work item c; lanes (threads) 0..26 of the caller fill nbr[27].
template<class T> __device__ __forceinline__ bool load_chunk(const DevState<T>& S,long long c,unsigned nc,unsigned nv,ChunkInfo<T>& ci,int* nbr,
                                                             int lane=-1)
{
    if(lane<0) lane=threadIdx.x;
    ci.s=S.chunk_start[c];
    ci.e=(c+1<nc)?S.chunk_start[c+1]:(int)nv;
    ci.gb=(long long)(S.keys[ci.s]>>6);
    ci.scene=scene_of_block(S.scene_block_base,S.n_scenes,ci.gb);
    const SceneDev<T>& sc=S.scenes[ci.scene];
    long long lb=ci.gb-sc.block_base;
    ci.b[0]=(int)(lb%sc.nb[0]);lb/=sc.nb[0];ci.b[1]=(int)(lb%sc.nb[1]);ci.b[2]=(int)(lb/sc.nb[1]);
    if(lane<27){
        const int ox=lane%3-1,oy=(lane/3)%3-1,oz=lane/9-1;
        const long long g2=ci.gb+ox+(long long)sc.nb[0]*(oy+(long long)sc.nb[1]*oz);
        nbr[lane]=bit_set(S.bitmap,g2)?S.blockmap[g2]:-1;}
    return true;
}
// Tile node t (0..215) -> global node index, or -1 if its block is not active.
__device__ __forceinline__ long long tile_node(const int* nbr,int t)
{
    const int tx=t%TILE,ty=(t/TILE)%TILE,tz=t/(TILE*TILE);
    const int ox=(tx+3)/4-1,oy=(ty+3)/4-1,oz=(tz+3)/4-1;        // 0 -> -1, 1..4 -> 0, 5 -> +1
    const int idx=nbr[(ox+1)+3*(oy+1)+9*(oz+1)];
    if(idx<0) return -1;
    const int l=((tx+3)&3)|(((ty+3)&3)<<2)|(((tz+3)&3)<<4);
    return (long long)idx*64+l;
}
// Per-particle stencil data: tile coordinates of node c-1 and the weights along each axis.
template<class T> struct Stencil {
    int r[3];        // tile coordinate of the particle's cell (1..4)
    T w[3][3],dw[3][3];
};
template<class T> __device__ __forceinline__ void make_stencil(const SceneDev<T>& sc,const int* b,unsigned key,const T* X,Stencil<T>& st)
{
    const unsigned l=key&63u;
    const int lc[3]={(int)(l&3u),(int)((l>>2)&3u),(int)(l>>4)};
#pragma unroll
    for(int a=0;a<3;++a){
        st.r[a]=lc[a]+1;
        const int cell=4*b[a]+lc[a]-4;
        // x = (X - (center(c) - dx))/dx, evaluated in the same order as the reference
        const T center=fmul_rn<T>(add_rn<T>((T)cell,(T)0.5),sc.dx[a]);
        const T xe=sub_rn<T>(X[a],sub_rn<T>(center,sc.dx[a]));
        bspline_weights<T>(fmul_rn<T>(xe,sc.inv_dx[a]),sc.inv_dx[a],st.w[a],st.dw[a]);}
}
// Node centre of a grid node.
template<class T> __device__ __forceinline__ void node_center(const DevState<T>& S,const SceneDev<T>& sc,long long node,int blk,T* x)
{
    long long lb=(long long)S.active_gb[blk]-sc.block_base;
    const int bx=(int)(lb%sc.nb[0]);lb/=sc.nb[0];const int by=(int)(lb%sc.nb[1]),bz=(int)(lb/sc.nb[1]);
    const int l=(int)(node&63);
    const int c[3]={4*bx+(l&3)-4,4*by+((l>>2)&3)-4,4*bz+(l>>4)-4};
#pragma unroll
    for(int a=0;a<3;++a) x[a]=((T)c[a]+(T)0.5)*sc.dx[a];
}
template<class T> __device__ __forceinline__ bool inside_barrier(const SceneDev<T>& sc,int b,const T* x)
{return (x[0]-sc.bs[b][0])*sc.bn[b][0]+(x[1]-sc.bs[b][1])*sc.bn[b][1]+(x[2]-sc.bs[b][2])*sc.bn[b][2]<T(0);}

// Particle order inside a work item for the scatter kernels: the item's n particles are
// split into 32 runs of `stride` = ceil(n/32) consecutive (cell-sorted) particles, lane L
// walks run L, and the CTA's warps take successive positions inside the runs. Lanes of a
// warp therefore sit about n/32 particles apart, i.e. in different cells for a full
// block, and their shared atomics rarely hit the same node.
#define FOR_INTERLEAVED(n,jvar) \
    for(int q_=(int)(threadIdx.x>>5),st_=((n)+31)>>5;q_<st_;q_+=(int)(blockDim.x>>5)) \
        for(int jvar=(int)(threadIdx.x&31)*st_+q_,ok_=1;ok_;ok_=0) if(jvar<(n))

// ---------- per-scene reductions inside node kernels ----------
struct SceneRed {
    double sum[MAX_SCENES];
    unsigned long long mx[MAX_SCENES];
    unsigned long long cnt[MAX_SCENES];
};
__device__ __forceinline__ void red_init(SceneRed& R,int ns)
{for(int i=threadIdx.x;i<ns;i+=blockDim.x){R.sum[i]=0.;R.mx[i]=0ull;R.cnt[i]=0ull;}}
template<class TR> __device__ __forceinline__ TR warp_sum(TR v){for(int o=16;o>0;o>>=1) v+=__shfl_xor_sync(0xffffffffu,v,o);return v;}
template<class TR> __device__ __forceinline__ TR warp_max(TR v){for(int o=16;o>0;o>>=1){TR u=__shfl_xor_sync(0xffffffffu,v,o);v=u>v?u:v;}return v;}
__device__ __forceinline__ unsigned long long dbits(double x){return (unsigned long long)__double_as_longlong(x);}
__device__ __forceinline__ double bitsd(unsigned long long b){return __longlong_as_double((long long)b);}
// Flush the CTA's per-scene partials to the global accumulators, then let the last CTA
// (ticket) run `fin` for every scene; fin sees complete sums. Returns true in every
// thread of the last CTA.
template<class F> __device__ __forceinline__ bool red_finish(SceneRed& R,int ns,SceneAcc* acc,unsigned* ticket,F fin,bool use_sum,bool use_max,bool use_cnt)
{
    __syncthreads();
    for(int i=threadIdx.x;i<ns;i+=blockDim.x){
        if(use_sum&&R.sum[i]!=0.) atomicAdd(&acc[i].sum0,R.sum[i]);
        if(use_max&&R.mx[i]) atomicMax(&acc[i].max0,R.mx[i]);
        if(use_cnt&&R.cnt[i]) atomicAdd(&acc[i].count0,R.cnt[i]);}
    __threadfence();
    __shared__ bool last;
    __syncthreads();
    if(threadIdx.x==0) last=(atomicAdd(ticket,1u)==gridDim.x-1);
    __syncthreads();
    if(!last) return false;
    __threadfence();
    for(int i=threadIdx.x;i<ns;i+=blockDim.x){
        volatile SceneAcc* a=acc+i;
        const double s=a->sum0;const unsigned long long m=a->max0,c=a->count0;
        a->sum0=0.;a->max0=0ull;a->count0=0ull;
        fin(i,s,bitsd(m),c);}
    __syncthreads();
    if(threadIdx.x==0) *ticket=0u;
    return true;
}

// A warp's contiguous share [b, b1) of nb node blocks.
struct WarpRange {
    int b,b1;
    __device__ __forceinline__ explicit WarpRange(int nb)
    {
        const int nw=(int)(gridDim.x*(blockDim.x>>5)),gw=(int)(blockIdx.x*(blockDim.x>>5)+(threadIdx.x>>5));
        const int per=(nb+nw-1)/nw;
        b=gw*per<nb?gw*per:nb;b1=b+per<nb?b+per:nb;
    }
};
// Exclusive prefix sum of one int per thread over the CTA (any blockDim up to 1024);
// *total receives the sum. Called by every thread.
__device__ __forceinline__ int cta_scan_int(int v,int* total)
{
    __shared__ int wsum[32];
    const int lane=threadIdx.x&31,w=threadIdx.x>>5,nw=(blockDim.x+31)>>5;
    int x=v;
#pragma unroll
    for(int o=1;o<32;o<<=1){const int y=__shfl_up_sync(0xffffffffu,x,o);if(lane>=o) x+=y;}
    if(lane==31) wsum[w]=x;
    __syncthreads();
    if(w==0){int t=lane<nw?wsum[lane]:0;
#pragma unroll
        for(int o=1;o<32;o<<=1){const int y=__shfl_up_sync(0xffffffffu,t,o);if(lane>=o) t+=y;}
        wsum[lane]=t;}
    __syncthreads();
    const int excl=x-v+(w>0?wsum[w-1]:0);
    *total=wsum[nw-1];
    __syncthreads();
    return excl;
}
// Last CTA of a convergence check (after its per-scene updates of S.cg): the list of the
// scenes that still iterate, for the next loop trip. One thread per scene (blockDim >=
// n_scenes); every thread of the CTA calls it.
template<class T> __device__ __forceinline__ void build_active_list(const DevState<T>& S)
{
    __syncthreads();
    const int i=threadIdx.x;
    int act=0,nc=0,nb=0;
    if(i<S.n_scenes&&!S.cg[i].done){const SceneRange r=S.srange[i];act=1;nc=r.c1-r.c0;nb=r.b1-r.b0;}
    int na,ct,bt;
    const int pos=cta_scan_int(act,&na),cp=cta_scan_int(nc,&ct),bp=cta_scan_int(nb,&bt);
    ActiveList* L=S.alist;
    if(act){L->scene[pos]=i;L->cpre[pos]=cp;L->bpre[pos]=bp;}
    if(i==0){L->n=na;L->cpre[na]=ct;L->bpre[na]=bt;}
}
// The list staged in shared memory by every CTA of a loop-trip kernel.
struct ListSmem { int n; int scene[MAX_SCENES]; int pre[MAX_SCENES+1]; };
__device__ __forceinline__ void load_active_list(const ActiveList* L,ListSmem& sm,bool blocks)
{
    const int n=L->n;
    for(int k=threadIdx.x;k<=n;k+=blockDim.x){
        if(k<n) sm.scene[k]=L->scene[k];
        sm.pre[k]=blocks?L->bpre[k]:L->cpre[k];}
    if(threadIdx.x==0) sm.n=n;
    __syncthreads();
}
// Position j in the list with pre[j] <= w < pre[j+1] (w < pre[n]).
__device__ __forceinline__ int list_find(const ListSmem& sm,int w)
{
    int lo=0,hi=sm.n-1;
    while(lo<hi){const int mid=(lo+hi+1)>>1;if(sm.pre[mid]<=w) lo=mid;else hi=mid-1;}
    return lo;
}

// =====================================================================================
// K3: plasticity + P2G. Per particle: Precompute (MPM_Constitutive_Model.cpp:32-51,
// called at MPM_Example.cpp:563-571), then the scatter of m, m v (Rasterize,
// MPM_Example.cpp:520-537) and f = sum_p (m_p g w - V0 P Fe^T grad w) (Apply_Explicit_Force,
// MPM_Example.cpp:757-784). Reads the old particle buffer through the sort permutation and
// writes the new one, cell-ordered inside every work item, with its keys and the CG cache.
// =====================================================================================
// Shared-memory bytes of one P2G / Hessian CTA: the warps' private tiles and, for P2G, the
// cell order of a work item of up to `chunk` particles (per-warp cell counts, slot -> item
// map, item cells).
template<class T> __host__ __device__ constexpr int p2g_tile_bytes(){return (XFER_THREADS/32)*7*TILE_S*(int)sizeof(T);}
__host__ __device__ constexpr int order_bytes(int chunk){return (XFER_THREADS/32)*64*4+((chunk*3+15)&~15);}
template<class T> __host__ __device__ constexpr int p2g_smem_bytes(int chunk){return p2g_tile_bytes<T>()+order_bytes(chunk);}
template<class T> constexpr int hess_smem_bytes(){return (XFER_THREADS/32)*3*TILE_S*(int)sizeof(T)+3*TILE_S*(int)sizeof(T);}
template<class T> constexpr int hess_warp_smem_bytes(){return (XFER_THREADS/32)*6*TILE_S*(int)sizeof(T);}

// Scatter order of a block's 64 cells: by the shared-memory bank of the cell's tile address
// (tile_addr mod 32), then by cell index. With TSZ = 40 every bank holds exactly two cells,
// so cells of even rank have 32 distinct banks, and so do cells of odd rank. A warp's lanes
// sit about two cells apart in this order (a full block has 8 particles per cell and the
// lanes are chunk/32 particles apart), so their tile addresses, and for every stencil
// offset the addresses of their nodes, fall in distinct banks.
__device__ __forceinline__ unsigned char cell_rank_of(int l)
{
    const int b=tile_addr(l&3,(l>>2)&3,l>>4)&31;
    int k=0;
    for(int m=0;m<64;++m){const int bm=tile_addr(m&3,(m>>2)&3,m>>4)&31;k+=(bm<b||(bm==b&&m<l));}
    return (unsigned char)k;
}

// Storage order of a work item. Pass q of a warp gives lane L the cell-ordered slot
// k = L*stride + q (stride = ceil(np/32)), so the lanes of a warp sit about two cells
// apart. Slot (q, L) is stored at position run[q] + L, where run[q] counts the valid slots
// of the passes before q (the valid lanes of a pass are a prefix of the warp): a warp's
// loads and stores of one pass are contiguous. Called by warp 0; run has stride+1 entries
// (stride <= 128 for work items of up to 4096 particles).
__device__ __forceinline__ void chunk_runs(int np,int stride,int* run)
{
    const int lane=threadIdx.x&31;
    int c[4],tot=0;
#pragma unroll
    for(int u=0;u<4;++u){
        const int q=4*lane+u;const int r=np-q;
        c[u]=(q<stride&&r>0)?min(32,(r+stride-1)/stride):0;tot+=c[u];}
    int incl=tot;
#pragma unroll
    for(int o=1;o<32;o<<=1){const int v=__shfl_up_sync(0xffffffffu,incl,o);if(lane>=o) incl+=v;}
    int acc=incl-tot;
#pragma unroll
    for(int u=0;u<4;++u){const int q=4*lane+u;if(q<=stride) run[q]=acc;acc+=c[u];}
}

// Stable counting sort of a work item's particles by the scatter rank of their cell (the
// low 6 key bits through crank): on return inv[k] is the item position of the k-th
// particle in (rank, item position) order, and cellv[j] the cell of item position j. Warp
// w owns the item positions [w*seg, (w+1)*seg); a first pass counts ranks per warp, a warp
// scan turns the counts into (rank, warp)-major offsets, and a second pass places every
// particle. The particles of a block keep their order from one substep to the next (the
// block sort is stable), so writing the new buffer in this order makes the chunk
// rank-sorted for the Hessian and G2P of this substep and nearly so for the next P2G.
__device__ __forceinline__ void chunk_cell_order(const unsigned* keys,int s,int np,const unsigned char* crank,int (*cnt)[64],unsigned short* inv,unsigned char* cellv)
{
    const int lane=threadIdx.x&31,warp=threadIdx.x>>5,nw=blockDim.x>>5;
    for(int t=threadIdx.x;t<nw*64;t+=blockDim.x) (&cnt[0][0])[t]=0;
    __syncthreads();
    const int seg=(np+nw-1)/nw,b0=warp*seg,b1=min(np,b0+seg);
    const unsigned below=lane_bits_below();
    for(int g=b0;g<b1;g+=32){
        const int j=g+lane;const bool ok=j<b1;
        const unsigned cell=ok?(keys[s+j]&63u):0u;
        if(ok) cellv[j]=(unsigned char)cell;
        const unsigned rk=ok?(unsigned)crank[cell]:64u+lane;
        const unsigned peers=__match_any_sync(0xffffffffu,rk);
        if(ok&&(peers&below)==0) cnt[warp][rk]+=__popc(peers);
        __syncwarp();}
    __syncthreads();
    if(warp==0){
        const int c0=2*lane,c1=2*lane+1;
        int t0=0,t1=0;
        for(int w=0;w<nw;++w){t0+=cnt[w][c0];t1+=cnt[w][c1];}
        int incl=t0+t1;
#pragma unroll
        for(int o=1;o<32;o<<=1){const int u=__shfl_up_sync(0xffffffffu,incl,o);if(lane>=o) incl+=u;}
        int o0=incl-(t0+t1),o1=o0+t0;
        for(int w=0;w<nw;++w){
            const int a=cnt[w][c0],b=cnt[w][c1];
            cnt[w][c0]=o0;o0+=a;cnt[w][c1]=o1;o1+=b;}}
    __syncthreads();
    for(int g=b0;g<b1;g+=32){
        const int j=g+lane;const bool ok=j<b1;
        const unsigned rk=ok?(unsigned)crank[cellv[j]]:64u+lane;
        const unsigned peers=__match_any_sync(0xffffffffu,rk);
        if(ok) inv[cnt[warp][rk]+__popc(peers&below)]=(unsigned short)j;
        __syncwarp();
        if(ok&&(peers&below)==0) cnt[warp][rk]+=__popc(peers);
        __syncwarp();}
    __syncthreads();
}

// G[3a+k] = sum_n s_a(n) d_k w(n) over the 27 stencil nodes, for a tile s[3][TILE_N]. The
// weights are separable, w = wx wy wz: the z sums of wz s_a and dwz s_a come first, then
// each (x, y) pair adds them with dwx wy, wx dwy and wx wy.
// FP32: components 0 and 1 of the staged vector as packed pairs, component 2 scalar.
__device__ __forceinline__ void gather_grad(const Stencil<float>& st,const float (*s)[TILE_S],float* G)
{
    float2 g03=make_float2(0.f,0.f),g14=g03,g25=g03;
    float g6=0.f,g7=0.f,g8=0.f;
    const int tb=tile_addr(st.r[0]-1,st.r[1]-1,st.r[2]-1);
#pragma unroll
    for(int ox=0;ox<3;++ox)
#pragma unroll
    for(int oy=0;oy<3;++oy){
        float2 t01=make_float2(0.f,0.f),u01=t01;
        float t2=0.f,u2=0.f;
#pragma unroll
        for(int oz=0;oz<3;++oz){
            const float wz=st.w[2][oz],dz=st.dw[2][oz];
            const int n=tb+tile_addr(ox,oy,oz);
            const float2 s01=make_float2(s[0][n],s[1][n]);
            const float s2=s[2][n];
            t01=pfma(pdup(wz),s01,t01);u01=pfma(pdup(dz),s01,u01);
            t2=fmaf(wz,s2,t2);u2=fmaf(dz,s2,u2);}
        const float dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
        g03=pfma(pdup(dxy),t01,g03);g14=pfma(pdup(xdy),t01,g14);g25=pfma(pdup(wxy),u01,g25);
        g6=fmaf(dxy,t2,g6);g7=fmaf(xdy,t2,g7);g8=fmaf(wxy,u2,g8);}
    G[0]=g03.x;G[3]=g03.y;G[1]=g14.x;G[4]=g14.y;G[2]=g25.x;G[5]=g25.y;G[6]=g6;G[7]=g7;G[8]=g8;
}
template<class T> __device__ __forceinline__ void gather_grad(const Stencil<T>& st,const T (*s)[TILE_S],T* G)
{
#pragma unroll
    for(int k=0;k<9;++k) G[k]=T(0);
    const int tb=tile_addr(st.r[0]-1,st.r[1]-1,st.r[2]-1);
#pragma unroll
    for(int ox=0;ox<3;++ox)
#pragma unroll
    for(int oy=0;oy<3;++oy){
        T t[3]={T(0),T(0),T(0)},u[3]={T(0),T(0),T(0)};
#pragma unroll
        for(int oz=0;oz<3;++oz){
            const T wz=st.w[2][oz],dz=st.dw[2][oz];
            const int n=tb+tile_addr(ox,oy,oz);
#pragma unroll
            for(int a=0;a<3;++a){const T sa=s[a][n];t[a]+=wz*sa;u[a]+=dz*sa;}}
        const T dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
#pragma unroll
        for(int a=0;a<3;++a){G[3*a]+=dxy*t[a];G[3*a+1]+=xdy*t[a];G[3*a+2]+=wxy*u[a];}}
}

// Conflict-free rounds for a warp's scatter into its private tile. Lanes whose particles
// share a cell are spread over successive rounds, so inside a round the lanes' cells
// differ and, for any one stencil offset, so do their nodes: one offset's read-add-write
// is conflict free. Two lanes can still reach the same node through different offsets,
// so each offset's update is ordered before the next one's with __syncwarp over the
// round's lanes. (This replaced shared-memory float atomics on one CTA-wide tile: C1's
// P2G went from ~0.2 to 0.11 ms per launch.)
struct ScatterRounds {
    int rank,rounds;
    __device__ __forceinline__ ScatterRounds(bool valid,unsigned cell)
    {
        const unsigned peers=__match_any_sync(0xffffffffu,valid?cell:(64u+(threadIdx.x&31)));
        rank=__popc(peers&lane_bits_below());
        rounds=(int)__reduce_max_sync(0xffffffffu,(unsigned)rank)+1;
    }
};

// One pass of a work item's particles through P2G: pass qi gives lane L the cell-ordered
// particle L*stride + qi (item position inv[k] in the sorted order, read through the sort
// permutation from the old buffer), which is stored at position run[qi] + L of the new
// buffer. Precompute (plasticity), the new buffer's state, cache and key, then the scatter
// of m, m v and f into the warp's tile in rounds of lanes in distinct cells. Called by
// every lane of the warp.
template<class P> __device__ __forceinline__ void p2g_pass(const DevState<typename P::T>& S,const SceneDev<typename P::T>& sc,
    const ChunkInfo<typename P::T>& ci,const int* run,const unsigned short* inv,const unsigned char* cellv,int qi,int stride,int np,
    typename P::T (*tile)[TILE_S])
{
    using T=typename P::T; using TS=typename P::TS;
    // cell-ordered slot k: item position inv[k] in, position run[qi] + lane out
    const int k=(int)(threadIdx.x&31)*stride+qi;
    const bool valid=k<np;
    const int i=ci.s+run[qi]+(int)(threadIdx.x&31);
    T A[9],X[3],V[3],m=T(0);
    Stencil<T> st;
    unsigned cell=0;
    if(valid){
        const long long pc=S.pcap;
        const int jj=inv[k];
        const int src=S.perm[ci.s+jj];
        const T* Pin=S.pcur;T* Pout=S.pnxt;
        T F[9];
#pragma unroll
        for(int a=0;a<3;++a){X[a]=Pin[(FX+a)*pc+src];V[a]=Pin[(FV+a)*pc+src];}
#pragma unroll
        for(int k=0;k<9;++k) F[k]=Pin[(FF+k)*pc+src];
        T Jp=Pin[FJP*pc+src];
        m=Pin[FM*pc+src];
        const T V0=Pin[FV0*pc+src],lam0=Pin[FLAM0*pc+src],mu0=Pin[FMU0*pc+src];
        T R[9],lam,mu,Je;
        if(sc.eos){
            // EOS fluid (MPM_Example.cpp:737-738): no constitutive update; the
            // density is the Jp slot. The CG's coefficient V0 k gamma rho^(gamma-1)
            // goes to the lambda cache slot, the explicit one V0/rho k rho^(gamma-1)
            // to the mu slot.
            const T pw=tpow(Jp,sc.eos_gamma-T(1));
            lam=V0*sc.bulk*sc.eos_gamma*pw;mu=V0/Jp*sc.bulk*pw;Je=T(1);
#pragma unroll
            for(int k=0;k<9;++k) R[k]=(k%4==0)?T(1):T(0);}
        else precompute<T,TS>(F,Jp,lam0,mu0,sc.plastic,sc.hardening,sc.cy,sc.sy,sc.hmax,R,lam,mu,Je);
#pragma unroll
        for(int a=0;a<3;++a){Pout[(FX+a)*pc+i]=X[a];Pout[(FV+a)*pc+i]=V[a];}
#pragma unroll
        for(int k=0;k<9;++k){Pout[(FF+k)*pc+i]=F[k];S.cache[(CR+k)*pc+i]=R[k];}
        Pout[FJP*pc+i]=Jp;Pout[FM*pc+i]=m;Pout[FV0*pc+i]=V0;Pout[FLAM0*pc+i]=lam0;Pout[FMU0*pc+i]=mu0;
        S.cache[CLAM*pc+i]=lam;S.cache[CMU*pc+i]=mu;
        S.pid_nxt[i]=S.pid_cur[src];S.scn_nxt[i]=S.scn_cur[src];
        if(sc.eos){
            // f += coefficient grad w, i.e. A = -coefficient I
#pragma unroll
            for(int k=0;k<9;++k) A[k]=(k%4==0)?-mu:T(0);}
        else{
            // V0 P Fe^T
            T Pk[9];stress_P(F,R,lam,mu,Je,Pk);mat_mul_bt(Pk,F,A);
#pragma unroll
            for(int k=0;k<9;++k) A[k]*=V0;}
        cell=cellv[jj];
        const unsigned key=((unsigned)ci.gb<<6)|cell;
        S.keys[i]=key;
        make_stencil(sc,ci.b,key,X,st);}
    const ScatterRounds R(valid,cell);
    for(int r=0;r<R.rounds;++r){
        const unsigned rmask=__ballot_sync(0xffffffffu,valid&&R.rank==r);
        if(valid&&R.rank==r){
            const int tb=tile_addr(st.r[0]-1,st.r[1]-1,st.r[2]-1);
            const T mv0=m*V[0],mv1=m*V[1],mv2=m*V[2];
            const T mg0=sc.gravity[0]*m,mg1=sc.gravity[1]*m,mg2=sc.gravity[2]*m;
#pragma unroll
            for(int ox=0;ox<3;++ox)
#pragma unroll
            for(int oy=0;oy<3;++oy){
                // at this (x, y): w = wxy wz and f_a = m g_a w - sum_k A_ak grad_k w
                // = al_a wz - be_a dwz
                const T dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
                const T cm=m*wxy,cv0=mv0*wxy,cv1=mv1*wxy,cv2=mv2*wxy;
                const T al0=mg0*wxy-(A[0]*dxy+A[1]*xdy),al1=mg1*wxy-(A[3]*dxy+A[4]*xdy),al2=mg2*wxy-(A[6]*dxy+A[7]*xdy);
                const T be0=A[2]*wxy,be1=A[5]*wxy,be2=A[8]*wxy;
                if constexpr(sizeof(T)==4){
                    // channels (0, 1), (2, 3) and (4, 5) as packed pairs, channel 6 scalar:
                    // each lane of a pair is the same fused multiply-add as the scalar form
                    const float2 c01=make_float2(cm,cv0),c23=make_float2(cv1,cv2);
                    const float2 al45=make_float2(al0,al1),nbe45=make_float2(-be0,-be1);
#pragma unroll
                    for(int oz=0;oz<3;++oz){
                        const T wz=st.w[2][oz],dz=st.dw[2][oz];
                        const int t=tb+tile_addr(ox,oy,oz);
                        const float2 q01=pfma(c01,pdup(wz),make_float2(tile[0][t],tile[1][t]));
                        const float2 q23=pfma(c23,pdup(wz),make_float2(tile[2][t],tile[3][t]));
                        const float2 q45=pfma(nbe45,pdup(dz),pfma(al45,pdup(wz),make_float2(tile[4][t],tile[5][t])));
                        tile[0][t]=q01.x;tile[1][t]=q01.y;tile[2][t]=q23.x;tile[3][t]=q23.y;
                        tile[4][t]=q45.x;tile[5][t]=q45.y;
                        tile[6][t]=tfma(-be2,dz,tfma(al2,wz,tile[6][t]));
                        __syncwarp(rmask);}}
                else{
#pragma unroll
                    for(int oz=0;oz<3;++oz){
                        const T wz=st.w[2][oz],dz=st.dw[2][oz];
                        const int t=tb+tile_addr(ox,oy,oz);
                        tile[0][t]=tfma(cm,wz,tile[0][t]);
                        tile[1][t]=tfma(cv0,wz,tile[1][t]);tile[2][t]=tfma(cv1,wz,tile[2][t]);tile[3][t]=tfma(cv2,wz,tile[3][t]);
                        // two fused multiply-adds per channel: tile + al wz - be dz
                        tile[4][t]=tfma(-be0,dz,tfma(al0,wz,tile[4][t]));
                        tile[5][t]=tfma(-be1,dz,tfma(al1,wz,tile[5][t]));
                        tile[6][t]=tfma(-be2,dz,tfma(al2,wz,tile[6][t]));
                        __syncwarp(rmask);}}}}
        __syncwarp();}
}

// The flush of a warp's (or the CTA's summed) P2G tile: one vector atomic per touched node
// and channel group.
template<class T> __device__ __forceinline__ void p2g_flush_node(const DevState<T>& S,const int* nbr,int t,const T* v)
{
    if(v[0]==T(0)&&v[4]==T(0)&&v[5]==T(0)&&v[6]==T(0)) return;
    const long long node=tile_node(nbr,t);
    if(node<0){atomicOr(&S.ctr->error,ERR_CAPACITY);return;}
    atomic_add_v3(S.gv+node,v[1],v[2],v[3],v[0]);
    atomic_add_v3(S.gf+node,v[4],v[5],v[6],T(0));
}
// Removed particles (slots >= n_valid after the sort) are carried to the new buffer as is.
template<class T> __device__ __forceinline__ void p2g_copy_removed(const DevState<T>& S,unsigned nv)
{
    const long long pc=S.pcap;
    for(long long i=(long long)nv+blockIdx.x*(long long)blockDim.x+threadIdx.x;i<S.n_total;i+=(long long)gridDim.x*blockDim.x){
        const int src=S.perm[i];
        for(int k=0;k<NB_FIELDS;++k) S.pnxt[k*pc+i]=S.pcur[k*pc+src];
        S.pid_nxt[i]=S.pid_cur[src];S.scn_nxt[i]=S.scn_cur[src];}
}

// Work items handled by the whole CTA: the four warps sort the item's particles by cell
// together, take its passes in turn into their own tiles, and the tiles are summed at the
// flush.
template<class P,int MINB> __global__ void __launch_bounds__(XFER_THREADS,MINB) k_p2g(DevState<typename P::T> S)
{
    pdl_enter();
    using T=typename P::T;
    constexpr int NW=XFER_THREADS/32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T (*acc)[7][TILE_S]=reinterpret_cast<T (*)[7][TILE_S]>(smem_raw);   // [warp][channel][node]
    int (*ocnt)[64]=reinterpret_cast<int (*)[64]>(smem_raw+p2g_tile_bytes<T>());
    unsigned short* inv=reinterpret_cast<unsigned short*>(smem_raw+p2g_tile_bytes<T>()+NW*64*4);
    unsigned char* cellv=reinterpret_cast<unsigned char*>(inv+S.chunk);
    __shared__ unsigned char crank[64];
    if(threadIdx.x<64) crank[threadIdx.x]=cell_rank_of(threadIdx.x);   // read after the next barrier
    __shared__ int nbr[27];
    __shared__ int run[129];
    const int warp=threadIdx.x>>5;
    const unsigned nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap),nv=S.ctr->n_valid;
    for(long long c=blockIdx.x;c<nc;c+=gridDim.x){
        ChunkInfo<T> ci;
        load_chunk(S,c,nc,nv,ci,nbr);
        const int np=ci.e-ci.s,stride=(np+31)>>5;
        if(np>S.chunk){if(threadIdx.x==0) atomicOr(&S.ctr->error,ERR_CAPACITY);continue;}   // uniform
        if(warp==0) chunk_runs(np,stride,run);        // read after the barriers in chunk_cell_order
        for(int t=threadIdx.x;t<NW*7*TILE_S;t+=blockDim.x) (&acc[0][0][0])[t]=T(0);
        chunk_cell_order(S.keys,ci.s,np,crank,ocnt,inv,cellv);
        const SceneDev<T>& sc=S.scenes[ci.scene];
        for(int qi=warp;qi<stride;qi+=NW) p2g_pass<P>(S,sc,ci,run,inv,cellv,qi,stride,np,acc[warp]);
        __syncthreads();
        for(int t=threadIdx.x;t<TILE_N;t+=blockDim.x){
            const int ta=tile_addr(t);
            T v[7];
#pragma unroll
            for(int ch=0;ch<7;++ch){T a=T(0);
#pragma unroll
                for(int w=0;w<NW;++w) a+=acc[w][ch][ta];
                v[ch]=a;}
            p2g_flush_node(S,nbr,t,v);}
        __syncthreads();
    }
    p2g_copy_removed(S,nv);
}

// Full permutation of the particle state (first grid build, before any P2G).
template<class T> __global__ void __launch_bounds__(256) k_permute(DevState<T> S)
{
    const long long pc=S.pcap;
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<S.n_total;i+=(long long)gridDim.x*blockDim.x){
        const int src=S.perm[i];
        for(int k=0;k<NB_FIELDS;++k) S.pnxt[k*pc+i]=S.pcur[k*pc+src];
        S.pid_nxt[i]=S.pid_cur[src];S.scn_nxt[i]=S.scn_cur[src];}
}

// Clears the accumulated node channels and records each scene's range in the work-item
// list and in the active-block list (SceneRange; the ranges were zeroed before the key pass).
template<class T> __global__ void __launch_bounds__(256) k_clear_nodes(DevState<T> S)
{
    pdl_enter();
    const long long na=(long long)min(S.ctr->n_active,(unsigned)S.block_cap);
    const long long nn=na*64;
    const long long t0=blockIdx.x*(long long)blockDim.x+threadIdx.x,stride=(long long)gridDim.x*blockDim.x;
    const V4<T> z={T(0),T(0),T(0),T(0)};
    for(long long n=t0;n<nn;n+=stride){S.gv[n]=z;S.gf[n]=z;}
    const long long nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap);
    auto chunk_scene=[&](long long c){return scene_of_block(S.scene_block_base,S.n_scenes,(long long)(S.keys[S.chunk_start[c]]>>6));};
    for(long long c=t0;c<nc;c+=stride){
        const int sc=chunk_scene(c);
        if(c==0||chunk_scene(c-1)!=sc) S.srange[sc].c0=(int)c;
        if(c+1==nc||chunk_scene(c+1)!=sc) S.srange[sc].c1=(int)(c+1);}
    for(long long b=t0;b<na;b+=stride){
        const int sc=S.active_scene[b];
        if(b==0||S.active_scene[b-1]!=sc) S.srange[sc].b0=(int)b;
        if(b+1==na||S.active_scene[b+1]!=sc) S.srange[sc].b1=(int)(b+1);}
}

// Mass-only P2G for the first-touch volumes (MPM_Driver::Initialize -> Rasterize).
template<class T> __global__ void __launch_bounds__(XFER_THREADS) k_p2g_mass(DevState<T> S)
{
    __shared__ T acc[TILE_S];
    __shared__ int nbr[27];
    const unsigned nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap),nv=S.ctr->n_valid;
    for(long long c=blockIdx.x;c<nc;c+=gridDim.x){
        ChunkInfo<T> ci;load_chunk(S,c,nc,nv,ci,nbr);
        for(int t=threadIdx.x;t<TILE_S;t+=blockDim.x) acc[t]=T(0);
        __syncthreads();
        const SceneDev<T>& sc=S.scenes[ci.scene];
        const int np=ci.e-ci.s;
        FOR_INTERLEAVED(np,j){
            const int i=ci.s+j;
            const long long pc=S.pcap;
            T X[3];for(int a=0;a<3;++a) X[a]=S.pcur[(FX+a)*pc+i];
            const T m=S.pcur[FM*pc+i];
            Stencil<T> st;make_stencil(sc,ci.b,S.keys[i],X,st);
            for(int ox=0;ox<3;++ox) for(int oy=0;oy<3;++oy) for(int oz=0;oz<3;++oz){
                const int t=tile_addr(st.r[0]+ox-1,st.r[1]+oy-1,st.r[2]+oz-1);
                atomicAdd(&acc[t],st.w[0][ox]*st.w[1][oy]*st.w[2][oz]*m);}}
        __syncthreads();
        for(int t=threadIdx.x;t<TILE_N;t+=blockDim.x){
            const int ta=tile_addr(t);
            if(acc[ta]==T(0)) continue;
            const long long node=tile_node(nbr,t);
            if(node<0){atomicOr(&S.ctr->error,ERR_CAPACITY);continue;}
            atomicAdd(&S.gv[node].w,acc[ta]);}
        __syncthreads();
    }
}
// Process_Waiting_Particles (MPM_Example.cpp:827-840): V0 = m_p/(sum_i w_ip m_i/dx^3)
// for particles whose V0 is not positive.
template<class T> __global__ void __launch_bounds__(XFER_THREADS) k_init_volume(DevState<T> S)
{
    __shared__ T tm[TILE_S];
    __shared__ int nbr[27];
    const unsigned nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap),nv=S.ctr->n_valid;
    for(long long c=blockIdx.x;c<nc;c+=gridDim.x){
        ChunkInfo<T> ci;load_chunk(S,c,nc,nv,ci,nbr);
        __syncthreads();
        for(int t=threadIdx.x;t<TILE_N;t+=blockDim.x){const long long node=tile_node(nbr,t);tm[tile_addr(t)]=node<0?T(0):S.gv[node].w;}
        __syncthreads();
        const SceneDev<T>& sc=S.scenes[ci.scene];
        for(int i=ci.s+threadIdx.x;i<ci.e;i+=blockDim.x){
            const long long pc=S.pcap;
            if(S.pcur[FV0*pc+i]>T(0)) continue;
            T X[3];for(int a=0;a<3;++a) X[a]=S.pcur[(FX+a)*pc+i];
            Stencil<T> st;make_stencil(sc,ci.b,S.keys[i],X,st);
            T density=T(0);
            for(int ox=0;ox<3;++ox) for(int oy=0;oy<3;++oy) for(int oz=0;oz<3;++oz){
                const int t=tile_addr(st.r[0]+ox-1,st.r[1]+oy-1,st.r[2]+oz-1);
                density+=st.w[0][ox]*st.w[1][oy]*st.w[2][oz]*tm[t];}
            density*=T(1)/(sc.dx[0]*sc.dx[1]*sc.dx[2]);
            S.pcur[FV0*pc+i]=S.pcur[FM*pc+i]/density;}
        __syncthreads();
    }
}

// =====================================================================================
// K4: grid update, one thread per node. Interior where m>0 (Flag_Setup_Helper.h:25-35),
// v=mv/m (Velocity_Normalization_Helper.h:39-52), v*=v+dt/m f (Explicit_Force_Helper.h:
// 43-56), plane barriers in list order (Grid_Based_Collision_Helper.h:57-85), rhs=v*
// (MPM_RHS_Helper.h:39-50), x=v*, s=0, and the CG state reset. The last CTA sets each
// scene's tolerance max(abs, rel*max|v*|).
// =====================================================================================
template<class T> __global__ void __launch_bounds__(NODE_THREADS) k_grid_update(DevState<T> S)
{
    pdl_enter();
    __shared__ SceneRed R;
    red_init(R,S.n_scenes);
    __syncthreads();
    const long long nn=(long long)min(S.ctr->n_active,(unsigned)S.block_cap)*64;
    const V4<T> z={T(0),T(0),T(0),T(0)};
    for(long long n=blockIdx.x*(long long)blockDim.x+threadIdx.x;n<nn;n+=(long long)gridDim.x*blockDim.x){
        const int blk=(int)(n>>6);
        const int scene=S.active_scene[blk];
        const SceneDev<T>& sc=S.scenes[scene];
        const V4<T> a=S.gv[n];
        const T m=a.w;
        T vn=T(0);unsigned cnt=0;
        if(m>T(0)){
            const T inv=T(1)/m;
            const T v[3]={a.x*inv,a.y*inv,a.z*inv};
            const V4<T> f=S.gf[n];
            const T c=(T)(*S.dtp)/m;
            T vs[3]={v[0]+c*f.x,v[1]+c*f.y,v[2]+c*f.z};
            unsigned char proj=0;
            if(sc.n_barriers){
                T x[3];node_center(S,sc,n,blk,x);
                for(int b=0;b<sc.n_barriers;++b){
                    if(!inside_barrier(sc,b,x)) continue;
                    proj=(unsigned char)(sc.project!=0);
                    if(sc.bsticky[b]){vs[0]=vs[1]=vs[2]=T(0);continue;}
                    const T nx=sc.bn[b][0],ny=sc.bn[b][1],nz=sc.bn[b][2],mu=sc.bmu[b];
                    const T proj=vs[0]*nx+vs[1]*ny+vs[2]*nz;
                    if(proj<T(0)){
                        vs[0]-=nx*proj;vs[1]-=ny*proj;vs[2]-=nz*proj;
                        const T nv=mpm_sqrt(vs[0]*vs[0]+vs[1]*vs[1]+vs[2]*vs[2]);
                        if(-proj*mu<nv){const T k=proj*mu/nv;vs[0]+=vs[0]*k;vs[1]+=vs[1]*k;vs[2]+=vs[2]*k;}
                        else{vs[0]=vs[1]=vs[2]=T(0);}}}}
            S.gv[n]=V4<T>{v[0],v[1],v[2],m};
            S.gx[n]=V4<T>{vs[0],vs[1],vs[2],T(0)};
            S.gr[n]=V4<T>{vs[0],vs[1],vs[2],T(0)};
            S.gm[n]=m;S.gproj[n]=proj;
            vn=vs[0]*vs[0]+vs[1]*vs[1]+vs[2]*vs[2];cnt=1;}
        else{S.gv[n]=z;S.gx[n]=z;S.gr[n]=z;S.gm[n]=T(0);S.gproj[n]=0;}
        S.gs[n]=z;S.gf[n]=z;
        const double wmax=warp_max<double>((double)vn);
        const unsigned wc=warp_sum<unsigned>(cnt);
        if((threadIdx.x&31)==0){if(wmax>0.) atomicMax(&R.mx[scene],dbits(wmax));if(wc) atomicAdd(&R.cnt[scene],(unsigned long long)wc);}
    }
    red_finish(R,S.n_scenes,S.acc2,&S.ctr->ticket[0],[&](int i,double,double mx,unsigned long long cnt){
        const SceneDev<T>& sc=S.scenes[i];CGState& st=S.cg[i];
        st.tol=fmax(sc.cg_abs_tol,sc.cg_rel_tol*sqrt(mx));
        st.rho=0.;st.alpha=0.;st.beta=0.;st.residual=0.;st.iters=0;st.done=0;st.converged=0;st.n_interior=(int)cnt;
    },false,true,true);
}

// =====================================================================================
// K5: Hessian action q_raw = K s for every scene still iterating (MPM_CG_System::Force,
// MPM_CG_System.h:150-215): gather dF = (sum_i s_i grad w_i^T) Fe, dP = dP/dF:dF, scatter
// (V0 Fe dP^T)^T grad w_i. The gathered vector is x (FROM_X, for r = b - A x) or the new
// search direction s = r + beta s_old, formed on the fly from r and the old s.
// =====================================================================================
// One pass of a work item's particles through the Hessian product: pass qi gives lane L the
// cell-ordered particle L*stride + qi (stored by P2G at position run[qi] + L). It gathers
// G = sum_n s(n) grad w(n)^T from the staged vector tile sv, forms
// A = V0 Fe dP(dF = G Fe)^T, and scatters A^T grad w into the warp's private tile in rounds
// of lanes in distinct cells. Called by every lane of the warp.
// Requests into L2 the fields the Hessian reads for particle position i (its pass runs
// next), so that those loads wait on L2 rather than on DRAM.
template<class T> __device__ __forceinline__ void prefetch_hessian_particle(const DevState<T>& S,int i)
{
    const long long pc=S.pcap;
    auto pf=[](const void* p){asm volatile("prefetch.global.L2 [%0];"::"l"(p));};
#pragma unroll
    for(int a=0;a<3;++a) pf(S.pcur+(FX+a)*pc+i);
#pragma unroll
    for(int k=0;k<9;++k){pf(S.pcur+(FF+k)*pc+i);pf(S.cache+(CR+k)*pc+i);}
    pf(S.pcur+FV0*pc+i);pf(S.cache+CLAM*pc+i);pf(S.cache+CMU*pc+i);pf(S.keys+i);
}
template<class P> __device__ __forceinline__ void hessian_pass(const DevState<typename P::T>& S,const SceneDev<typename P::T>& sc,
    const ChunkInfo<typename P::T>& ci,const int* run,int qi,int stride,int np,const typename P::T (*sv)[TILE_S],
    typename P::T (*tile)[TILE_S],int qn=-1)
{
    using T=typename P::T;
    const int j=(int)(threadIdx.x&31)*stride+qi;
    const bool valid=j<np;
    const int i=ci.s+run[qi]+(int)(threadIdx.x&31);   // the position P2G stored slot j at
    if(qn>=0&&(int)(threadIdx.x&31)*stride+qn<np) prefetch_hessian_particle(S,ci.s+run[qn]+(int)(threadIdx.x&31));
    T A[9];
    Stencil<T> st;
    unsigned cell=0;
    if(valid){
        const long long pc=S.pcap;
        T X[3];
#pragma unroll
        for(int a=0;a<3;++a) X[a]=S.pcur[(FX+a)*pc+i];
        const unsigned key=S.keys[i];
        make_stencil(sc,ci.b,key,X,st);
        cell=key&63u;
        // G[3a+k] = sum_n s_a grad_k w_n, contracted over z first (separable weights)
        T G[9];
        gather_grad(st,sv,G);
        if(sc.eos){
            // EOS fluid (MPM_CG_System.h:102-107, 138-140): coefficient times
            // sum_i grad w_i . s_i on the diagonal, scattered as eos_scp grad w
            const T e=S.cache[CLAM*pc+i]*(G[0]+G[4]+G[8]);
#pragma unroll
            for(int k=0;k<9;++k) A[k]=(k%4==0)?e:T(0);}
        else{
            T F[9],Rm[9];
#pragma unroll
            for(int k=0;k<9;++k){F[k]=S.pcur[(FF+k)*pc+i];Rm[k]=S.cache[(CR+k)*pc+i];}
            const T lam=S.cache[CLAM*pc+i],mu=S.cache[CMU*pc+i],V0=S.pcur[FV0*pc+i];
            T dF[9],dP[9];
            mat_mul(G,F,dF);
            dP_dF(F,Rm,lam,mu,dF,dP);
            mat_mul_bt(F,dP,A);        // Fe dP^T
#pragma unroll
            for(int k=0;k<9;++k) A[k]*=V0;}}
    const ScatterRounds R(valid,cell);
    for(int r=0;r<R.rounds;++r){
        const unsigned rmask=__ballot_sync(0xffffffffu,valid&&R.rank==r);
        if(valid&&R.rank==r){
            const int tb=tile_addr(st.r[0]-1,st.r[1]-1,st.r[2]-1);
#pragma unroll
            for(int ox=0;ox<3;++ox)
#pragma unroll
            for(int oy=0;oy<3;++oy){
                // q_a = sum_k A[3k+a] grad_k w = al_a wz + be_a dwz at this (x, y)
                const T dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
                if constexpr(sizeof(T)==4){
                    // channels 0 and 1 as packed pairs, channel 2 scalar
                    const float2 al01=pfma(make_float2(A[0],A[1]),pdup(dxy),pmul(make_float2(A[3],A[4]),pdup(xdy)));
                    const float2 be01=pmul(make_float2(A[6],A[7]),pdup(wxy));
                    const T al2=tfma(A[2],dxy,A[5]*xdy),be2=A[8]*wxy;
#pragma unroll
                    for(int oz=0;oz<3;++oz){
                        const T wz=st.w[2][oz],dz=st.dw[2][oz];
                        const int t=tb+tile_addr(ox,oy,oz);
                        float2 q01=make_float2(tile[0][t],tile[1][t]);
                        q01=pfma(be01,pdup(dz),pfma(al01,pdup(wz),q01));
                        tile[0][t]=q01.x;tile[1][t]=q01.y;
                        tile[2][t]=tfma(be2,dz,tfma(al2,wz,tile[2][t]));
                        __syncwarp(rmask);}}
                else{
                    const T al0=A[0]*dxy+A[3]*xdy,al1=A[1]*dxy+A[4]*xdy,al2=A[2]*dxy+A[5]*xdy;
                    const T be0=A[6]*wxy,be1=A[7]*wxy,be2=A[8]*wxy;
#pragma unroll
                    for(int oz=0;oz<3;++oz){
                        const T wz=st.w[2][oz],dz=st.dw[2][oz];
                        const int t=tb+tile_addr(ox,oy,oz);
                        // two fused multiply-adds per channel: tile + al wz + be dz
                        tile[0][t]=tfma(be0,dz,tfma(al0,wz,tile[0][t]));
                        tile[1][t]=tfma(be1,dz,tfma(al1,wz,tile[1][t]));
                        tile[2][t]=tfma(be2,dz,tfma(al2,wz,tile[2][t]));
                        __syncwarp(rmask);}}}}
        __syncwarp();}
}

// The Hessian's two ways of taking work items, one kernel (the form is a launch argument,
// uniform over the grid):
// - CTA per item (HESS_CTA): the CTA's warps share one staged vector tile and take the
//   passes of the item in turn, each into its own accumulation tile; the tiles are summed
//   at the flush. Suits launches with few work items (one scene, or the last CG trips of a
//   batch, where one scene still iterates).
// - Warp per item (HESS_WARP): each warp takes whole work items on its own, with its own
//   staged vector and accumulation tiles, synchronised by __syncwarp only (no CTA barrier
//   inside the loop). Suits launches with many items per SM (the 64-scene batch: about
//   37,000); with few, one warp per item leaves SMs idle.
// - HESS_AUTO: per launch, a warp per item when the launch has at least as many work items
//   as warps can be resident (`warp_min`, set by the host from the SM count and the
//   occupancy variant), else a CTA per item (the count is known on the device: all items
//   for the first product, the iterating scenes' items for a loop trip).
constexpr int HESS_CTA=0, HESS_WARP=1, HESS_AUTO=2;
template<class T> constexpr int hess_kernel_smem_bytes(){return hess_smem_bytes<T>()>hess_warp_smem_bytes<T>()?hess_smem_bytes<T>():hess_warp_smem_bytes<T>();}
template<class P,bool FROM_X> __device__ __forceinline__ void stage_vector(const DevState<typename P::T>& S,const int* nbr,typename P::T beta,
    typename P::T (*sv)[TILE_S],int t0,int dt)
{
    using T=typename P::T;
    for(int t=t0;t<TILE_N;t+=dt){
        const long long node=tile_node(nbr,t);
        T a=T(0),b=T(0),d=T(0);
        if(node>=0){
            if(FROM_X){const V4<T> x=S.gx[node];a=x.x;b=x.y;d=x.z;}
            else{const V4<T> r=S.gr[node],so=S.gs[node];a=r.x+beta*so.x;b=r.y+beta*so.y;d=r.z+beta*so.z;}}
        const int ta=tile_addr(t);
        sv[0][ta]=a;sv[1][ta]=b;sv[2][ta]=d;}
}
template<class P,bool FROM_X,int MINB> __global__ void __launch_bounds__(XFER_THREADS,MINB) k_hessian(DevState<typename P::T> S,int form,long long warp_min)
{
    pdl_enter();
    using T=typename P::T;
    constexpr int NW=XFER_THREADS/32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int nbr_s[NW][27];
    __shared__ int run_s[NW][129];
    __shared__ ListSmem lsm;
    const int warp=threadIdx.x>>5,lane=threadIdx.x&31;
    const unsigned nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap),nv=S.ctr->n_valid;
    // the first product (FROM_X) covers every work item; a loop trip only the work items of
    // the scenes still iterating (the list the previous convergence check wrote)
    long long nwork=nc;
    if(!FROM_X){load_active_list(S.alist,lsm,false);nwork=lsm.pre[lsm.n];}
    auto item=[&](long long w){
        if(FROM_X) return w;
        const int j=list_find(lsm,(int)w);return S.srange[lsm.scene[j]].c0+(w-lsm.pre[j]);};
    if(form==HESS_AUTO) form=nwork>=warp_min?HESS_WARP:HESS_CTA;
    if(form==HESS_CTA){
        T (*q)[3][TILE_S]=reinterpret_cast<T (*)[3][TILE_S]>(smem_raw);                 // [warp][component][node]
        T (*sv)[TILE_S]=reinterpret_cast<T (*)[TILE_S]>(smem_raw+NW*3*TILE_S*sizeof(T)); // [component][node]
        int* nbr=nbr_s[0];int* run=run_s[0];
        for(long long w=blockIdx.x;w<nwork;w+=gridDim.x){
            ChunkInfo<T> ci;load_chunk(S,item(w),nc,nv,ci,nbr);
            if(S.cg[ci.scene].done) continue;    // uniform over the CTA
            // a work item longer than `chunk` only arises when the work-item capacity was
            // exceeded (ERR_CAPACITY is set); its run table would not fit: skip it (uniform)
            if(ci.e-ci.s>S.chunk) continue;
            const T beta=(T)S.cg[ci.scene].beta;
            if(warp==0) chunk_runs(ci.e-ci.s,(ci.e-ci.s+31)>>5,run);
            __syncthreads();
            stage_vector<P,FROM_X>(S,nbr,beta,sv,threadIdx.x,blockDim.x);
            for(int t=threadIdx.x;t<NW*3*TILE_S;t+=blockDim.x) (&q[0][0][0])[t]=T(0);
            __syncthreads();
            const SceneDev<T>& sc=S.scenes[ci.scene];
            const int np=ci.e-ci.s,stride=(np+31)>>5;
            for(int qi=warp;qi<stride;qi+=NW) hessian_pass<P>(S,sc,ci,run,qi,stride,np,sv,q[warp],qi+NW<stride?qi+NW:-1);
            __syncthreads();
            for(int t=threadIdx.x;t<TILE_N;t+=blockDim.x){
                const int ta=tile_addr(t);
                T v[3];
#pragma unroll
                for(int ch=0;ch<3;++ch){T a=T(0);
#pragma unroll
                    for(int w2=0;w2<NW;++w2) a+=q[w2][ch][ta];
                    v[ch]=a;}
                if(v[0]==T(0)&&v[1]==T(0)&&v[2]==T(0)) continue;
                const long long node=tile_node(nbr,t);
                if(node<0) continue;
                atomic_add_v3(S.gf+node,v[0],v[1],v[2],T(0));}
            __syncthreads();
        }
    }
    else{
        T (*q)[TILE_S]=reinterpret_cast<T (*)[TILE_S]>(smem_raw)+6*warp;   // [component][node], accumulated
        T (*sv)[TILE_S]=q+3;                                                 // [component][node], gathered
        int* nbr=nbr_s[warp];int* run=run_s[warp];
        for(long long w=(long long)blockIdx.x*NW+warp;w<nwork;w+=(long long)gridDim.x*NW){
            ChunkInfo<T> ci;load_chunk(S,item(w),nc,nv,ci,nbr,lane);
            if(S.cg[ci.scene].done) continue;    // uniform over the warp
            if(ci.e-ci.s>S.chunk) continue;       // capacity exceeded (see above)
            const T beta=(T)S.cg[ci.scene].beta;
            chunk_runs(ci.e-ci.s,(ci.e-ci.s+31)>>5,run);
            __syncwarp();
            stage_vector<P,FROM_X>(S,nbr,beta,sv,lane,32);
            for(int t=lane;t<3*TILE_S;t+=32) (&q[0][0])[t]=T(0);
            __syncwarp();
            const SceneDev<T>& sc=S.scenes[ci.scene];
            const int np=ci.e-ci.s,stride=(np+31)>>5;
            for(int qi=0;qi<stride;++qi) hessian_pass<P>(S,sc,ci,run,qi,stride,np,sv,q,qi+1<stride?qi+1:-1);
            __syncwarp();
            for(int t=lane;t<TILE_N;t+=32){
                const int ta=tile_addr(t);
                const T v0=q[0][ta],v1=q[1][ta],v2=q[2][ta];
                if(v0==T(0)&&v1==T(0)&&v2==T(0)) continue;
                const long long node=tile_node(nbr,t);
                if(node<0) continue;
                atomic_add_v3(S.gf+node,v0,v1,v2,T(0));}
            __syncwarp();
        }
    }
}

// Project (MPM_CG_System.h:220-225, intended semantics of Project_Helper.h:30-45).
template<class T> __device__ __forceinline__ bool projected(const DevState<T>& S,const SceneDev<T>& sc,long long n,int blk)
{
    if(!sc.project||sc.n_barriers==0) return false;
    T x[3];node_center(S,sc,n,blk,x);
    for(int b=0;b<sc.n_barriers;++b) if(inside_barrier(sc,b,x)) return true;
    return false;
}

// CG start: r = b - (x + dt^2/m K x), Project(r), then the first convergence check of the
// restated CG loop (iteration 0).
template<class P> __global__ void __launch_bounds__(NODE_THREADS) k_cg_start(DevState<typename P::T> S,unsigned long long cond,int use_cond)
{
    pdl_enter();
    using T=typename P::T; using TR=typename P::TR;
    __shared__ SceneRed R;
    red_init(R,S.n_scenes);
    __syncthreads();
    const int na=(int)min(S.ctr->n_active,(unsigned)S.block_cap);
    const T dtT=(T)(*S.dtp),dt2=dtT*dtT;
    const WarpRange wr(na);
    int scene=-1;double acc=0.,amax=0.;
    auto flush=[&](int sc){
        const double ws=warp_sum<double>(acc),wm=warp_max<double>(amax);
        if((threadIdx.x&31)==0){if(ws!=0.) atomicAdd(&R.sum[sc],ws);if(wm>0.) atomicMax(&R.mx[sc],dbits(wm));}
        acc=0.;amax=0.;};
    for(int blk=wr.b;blk<wr.b1;++blk){
        const int sb=S.active_scene[blk];
        if(sb!=scene){if(scene>=0) flush(scene);scene=sb;}
        T m[2];V4<T> x[2],b[2],k[2];unsigned char pj[2];
#pragma unroll
        for(int h=0;h<2;++h){const long long n=((long long)blk<<6)+h*32+(threadIdx.x&31);m[h]=S.gm[n];x[h]=S.gx[n];b[h]=S.gr[n];k[h]=S.gf[n];pj[h]=S.gproj[n];}
#pragma unroll
        for(int h=0;h<2;++h){
            const long long n=((long long)blk<<6)+h*32+(threadIdx.x&31);
            if(m[h]>T(0)){
                const T c=dt2/m[h];
                T r[3]={b[h].x-(c*k[h].x+x[h].x),b[h].y-(c*k[h].y+x[h].y),b[h].z-(c*k[h].z+x[h].z)};
                if(pj[h]) r[0]=r[1]=r[2]=T(0);       // Project, flagged by the grid update
                S.gr[n]=V4<T>{r[0],r[1],r[2],T(0)};
                acc+=(double)(TR)(r[0]*(r[0]*m[h])+r[1]*(r[1]*m[h])+r[2]*(r[2]*m[h]));
                const double cn=(double)(TR)(r[0]*r[0]+r[1]*r[1]+r[2]*r[2]);
                amax=cn>amax?cn:amax;}
            S.gf[n]=V4<T>{T(0),T(0),T(0),T(0)};}
    }
    if(scene>=0) flush(scene);
    __shared__ int any;
    if(threadIdx.x==0) any=0;
    const bool last=red_finish(R,S.n_scenes,S.acc,&S.ctr->ticket[1],[&](int i,double rr,double mx,unsigned long long){
        const SceneDev<T>& sc=S.scenes[i];CGState& st=S.cg[i];
        const double cn=sqrt(mx);
        const double eps=sizeof(T)==4?1.1920928955078125e-07:2.220446049250313e-16;
        st.residual=cn;
        if(cn<=st.tol&&(0>=sc.cg_min_iters||cn<eps)){st.done=1;st.converged=1;}
        else if(sc.cg_max_iters<=0){st.done=1;st.converged=0;atomicOr(&S.ctr->error,ERR_CG_NOT_CONVERGED);}
        else{st.rho=rr;st.beta=0.;atomicOr(&any,1);}
    },true,true,false);
    if(last) build_active_list(S);
    if(last&&threadIdx.x==0){
        S.ctr->any_active=any;S.ctr->loop_iters=0;
        if(use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond,any?1u:0u);}
}

// CG part 1: s = r + beta s_old (stored), q = s + dt^2/m K s, Project(q), <s,q>_M; the last
// CTA forms alpha = rho/<s,q>.
// A warp's share of the node blocks of the scenes in the list: a contiguous range of list
// blocks, so that the warp meets each scene once and streams whole blocks (64 nodes, two
// per lane). next() moves to list block bw (non-decreasing) and tells whether the scene
// changed; node(h) is the lane's h-th node (h = 0, 1) of that block.
struct WarpBlocks {
    int b,b1,j=0,scene=-1;long long base=0;
    __device__ __forceinline__ explicit WarpBlocks(const ListSmem& sm){const WarpRange r(sm.pre[sm.n]);b=r.b;b1=r.b1;}
    __device__ __forceinline__ bool next(const ListSmem& sm,const SceneRange* sr,int bw)
    {
        if(scene>=0&&bw<sm.pre[j+1]) return false;
        while(bw>=sm.pre[j+1]) ++j;
        scene=sm.scene[j];base=sr[scene].b0-sm.pre[j];
        return true;
    }
    __device__ __forceinline__ long long node(int bw,int h) const {return ((base+bw)<<6)+h*32+(threadIdx.x&31);}
};
template<class P> __global__ void __launch_bounds__(NODE_THREADS) k_cg_q(DevState<typename P::T> S)
{
    pdl_enter();
    using T=typename P::T; using TR=typename P::TR;
    __shared__ SceneRed R;
    __shared__ ListSmem lsm;
    red_init(R,S.n_scenes);
    load_active_list(S.alist,lsm,true);     // the scenes still iterating (its barrier orders red_init)
    const T dtT=(T)(*S.dtp),dt2=dtT*dtT;
    WarpBlocks wb(lsm);
    double acc=0.;T beta=T(0);
    auto flush=[&](int sc){const double ws=warp_sum<double>(acc);if((threadIdx.x&31)==0&&ws!=0.) atomicAdd(&R.sum[sc],ws);acc=0.;};
    for(int bw=wb.b;bw<wb.b1;++bw){
        const int prev=wb.scene;
        if(wb.next(lsm,S.srange,bw)){if(prev>=0) flush(prev);beta=(T)S.cg[wb.scene].beta;}
        T m[2];V4<T> r[2],so[2],k[2];unsigned char pj[2];
#pragma unroll
        for(int h=0;h<2;++h){const long long n=wb.node(bw,h);m[h]=S.gm[n];r[h]=S.gr[n];so[h]=S.gs[n];k[h]=S.gf[n];pj[h]=S.gproj[n];}
#pragma unroll
        for(int h=0;h<2;++h){
            if(!(m[h]>T(0))) continue;
            const long long n=wb.node(bw,h);
            const T s[3]={r[h].x+beta*so[h].x,r[h].y+beta*so[h].y,r[h].z+beta*so[h].z};
            const T c=dt2/m[h];
            T qv[3]={c*k[h].x+s[0],c*k[h].y+s[1],c*k[h].z+s[2]};
            if(pj[h]) qv[0]=qv[1]=qv[2]=T(0);
            S.gs[n]=V4<T>{s[0],s[1],s[2],T(0)};
            S.gf[n]=V4<T>{qv[0],qv[1],qv[2],T(0)};
            acc+=(double)(TR)(s[0]*(qv[0]*m[h])+s[1]*(qv[1]*m[h])+s[2]*(qv[2]*m[h]));}
    }
    if(wb.scene>=0) flush(wb.scene);
    red_finish(R,S.n_scenes,S.acc,&S.ctr->ticket[2],[&](int i,double sq,double,unsigned long long){
        CGState& st=S.cg[i];
        if(st.done) return;
        st.alpha=sq!=0.?st.rho/sq:(double)FLT_MAX;
    },true,false,false);
}

// CG part 2: x += alpha s, r -= alpha q (Interior only), clear q for the next Hessian
// action, then the convergence check: stop when max|r| <= tol (and iters >= min, or the
// norm is below epsilon) or at cg_max_iters; else beta = <r,r>/rho, rho = <r,r>.
template<class P> __global__ void __launch_bounds__(NODE_THREADS) k_cg_update(DevState<typename P::T> S,unsigned long long cond,int use_cond,int max_trips)
{
    pdl_enter();
    using T=typename P::T; using TR=typename P::TR;
    __shared__ SceneRed R;
    __shared__ ListSmem lsm;
    red_init(R,S.n_scenes);
    load_active_list(S.alist,lsm,true);
    WarpBlocks wb(lsm);
    double acc=0.,amax=0.;T alpha=T(0);
    auto flush=[&](int sc){
        const double ws=warp_sum<double>(acc),wm=warp_max<double>(amax);
        if((threadIdx.x&31)==0){if(ws!=0.) atomicAdd(&R.sum[sc],ws);if(wm>0.) atomicMax(&R.mx[sc],dbits(wm));}
        acc=0.;amax=0.;};
    for(int bw=wb.b;bw<wb.b1;++bw){
        const int prev=wb.scene;
        if(wb.next(lsm,S.srange,bw)){if(prev>=0) flush(prev);alpha=(T)S.cg[wb.scene].alpha;}
        T m[2];V4<T> s[2],qv[2],x[2],r[2];
#pragma unroll
        for(int h=0;h<2;++h){const long long n=wb.node(bw,h);m[h]=S.gm[n];s[h]=S.gs[n];qv[h]=S.gf[n];x[h]=S.gx[n];r[h]=S.gr[n];}
#pragma unroll
        for(int h=0;h<2;++h){
            const long long n=wb.node(bw,h);
            if(m[h]>T(0)){
                x[h].x=alpha*s[h].x+x[h].x;x[h].y=alpha*s[h].y+x[h].y;x[h].z=alpha*s[h].z+x[h].z;
                r[h].x=-alpha*qv[h].x+r[h].x;r[h].y=-alpha*qv[h].y+r[h].y;r[h].z=-alpha*qv[h].z+r[h].z;
                S.gx[n]=x[h];S.gr[n]=r[h];
                acc+=(double)(TR)(r[h].x*(r[h].x*m[h])+r[h].y*(r[h].y*m[h])+r[h].z*(r[h].z*m[h]));
                const double cn=(double)(TR)(r[h].x*r[h].x+r[h].y*r[h].y+r[h].z*r[h].z);
                amax=cn>amax?cn:amax;}
            S.gf[n]=V4<T>{T(0),T(0),T(0),T(0)};}
    }
    if(wb.scene>=0) flush(wb.scene);
    __shared__ int any;
    if(threadIdx.x==0) any=0;
    const bool last=red_finish(R,S.n_scenes,S.acc,&S.ctr->ticket[3],[&](int i,double rr,double mx,unsigned long long){
        const SceneDev<T>& sc=S.scenes[i];CGState& st=S.cg[i];
        if(st.done) return;
        st.iters+=1;
        const double cn=sqrt(mx);
        const double eps=sizeof(T)==4?1.1920928955078125e-07:2.220446049250313e-16;
        st.residual=cn;
        if(cn<=st.tol&&(st.iters>=sc.cg_min_iters||cn<eps)){st.done=1;st.converged=1;}
        else if(st.iters>=sc.cg_max_iters){st.done=1;st.converged=0;atomicOr(&S.ctr->error,ERR_CG_NOT_CONVERGED);}
        else{st.beta=rr/st.rho;st.rho=rr;atomicOr(&any,1);}
    },true,true,false);
    if(last) build_active_list(S);
    if(last&&threadIdx.x==0){
        S.ctr->loop_iters+=1;S.ctr->total_trips+=1;
        // every scene stops by its cg_max_iters; the trip cap is a second, global bound
        if(S.ctr->loop_iters>=max_trips) any=0;
        S.ctr->any_active=any;
        if(use_cond) cudaGraphSetConditional((cudaGraphConditionalHandle)cond,any?1u:0u);}
}

// =====================================================================================
// K7: G2P (Update_Particle_Velocities_And_Positions, MPM_Example.cpp:633-660): for nodes
// with w>0, V_pic = sum w v*, V_flip = V + sum w (v*-v), grad v = sum v* grad w^T;
// Fe += dt grad v Fe; V = flip V_flip + (1-flip) V_pic; X += dt V_pic; particles outside
// [dx/2, 1-dx/2]^3 are removed.
// =====================================================================================
template<class T,int MINB> __global__ void __launch_bounds__(XFER_THREADS,MINB) k_g2p(DevState<T> S)
{
    pdl_enter();
    __shared__ T tv[6][TILE_S];
    __shared__ int nbr[27];
    const unsigned nc=min(S.ctr->n_chunks,(unsigned)S.chunk_cap),nv=S.ctr->n_valid;
    for(long long c=blockIdx.x;c<nc;c+=gridDim.x){
        ChunkInfo<T> ci;load_chunk(S,c,nc,nv,ci,nbr);
        __syncthreads();
        for(int t=threadIdx.x;t<TILE_N;t+=blockDim.x){
            const long long node=tile_node(nbr,t);
            const int ta=tile_addr(t);
            if(node>=0){const V4<T> v=S.gv[node],x=S.gx[node];
                tv[0][ta]=v.x;tv[1][ta]=v.y;tv[2][ta]=v.z;tv[3][ta]=x.x;tv[4][ta]=x.y;tv[5][ta]=x.z;}
            else{for(int k=0;k<6;++k) tv[k][ta]=T(0);}}
        if(c+gridDim.x<nc){                 // the first particles of this CTA's next work item into L2
            const long long in=S.chunk_start[c+gridDim.x]+(long long)threadIdx.x;
            if(in<(long long)nv){
                auto pf=[](const void* p){asm volatile("prefetch.global.L2 [%0];"::"l"(p));};
#pragma unroll
                for(int k=0;k<15;++k) pf(S.pcur+(FX+k)*S.pcap+in);
                pf(S.keys+in);}}
        __syncthreads();
        const SceneDev<T>& sc=S.scenes[ci.scene];
        for(int i=ci.s+threadIdx.x;i<ci.e;i+=blockDim.x){
            const long long pc=S.pcap;
            if(i+(int)blockDim.x<ci.e){     // the thread's next particle into L2 (latency-bound on these loads)
                const int in=i+(int)blockDim.x;
                auto pf=[](const void* p){asm volatile("prefetch.global.L2 [%0];"::"l"(p));};
#pragma unroll
                for(int k=0;k<15;++k) pf(S.pcur+(FX+k)*pc+in);    // X, V, Fe
                pf(S.keys+in);}
            T X[3],V[3],F[9];
#pragma unroll
            for(int a=0;a<3;++a){X[a]=S.pcur[(FX+a)*pc+i];V[a]=S.pcur[(FV+a)*pc+i];}
#pragma unroll
            for(int k=0;k<9;++k) F[k]=S.pcur[(FF+k)*pc+i];
            Stencil<T> st;make_stencil(sc,ci.b,S.keys[i],X,st);
            // V_pic = sum w v*, the FLIP increment sum w (v* - v), grad v = sum v* grad w^T, contracted over z
            // first. Nodes with w = 0 (a particle exactly on a stencil edge) add nothing: their
            // weight and, along the same axis, the weight's derivative vanish together.
            T vp[3]={T(0),T(0),T(0)},vd[3]={T(0),T(0),T(0)};
            T G[9]={T(0),T(0),T(0),T(0),T(0),T(0),T(0),T(0),T(0)};
            const int tb=tile_addr(st.r[0]-1,st.r[1]-1,st.r[2]-1);
            if constexpr(sizeof(T)==4){
                // components 0 and 1 as packed pairs, component 2 scalar: each lane of a pair
                // is the same fused multiply-add (or subtraction) as the scalar form
                float2 vp01=make_float2(0.f,0.f),vd01=vp01,g0=vp01,g1=vp01,g2=vp01;   // g0 = (G[0], G[3]) ...
#pragma unroll
                for(int ox=0;ox<3;++ox)
#pragma unroll
                for(int oy=0;oy<3;++oy){
                    float2 ts01=make_float2(0.f,0.f),us01=ts01,to01=ts01;
                    float ts2=0.f,us2=0.f,to2=0.f;
#pragma unroll
                    for(int oz=0;oz<3;++oz){
                        const float wz=st.w[2][oz],dz=st.dw[2][oz];
                        const int t=tb+tile_addr(ox,oy,oz);
                        const float2 s01=make_float2(tv[3][t],tv[4][t]);
                        const float2 d01=__fadd2_rn(s01,make_float2(-tv[0][t],-tv[1][t]));
                        ts01=pfma(pdup(wz),s01,ts01);us01=pfma(pdup(dz),s01,us01);to01=pfma(pdup(wz),d01,to01);
                        const float s2=tv[5][t];
                        ts2=fmaf(wz,s2,ts2);us2=fmaf(dz,s2,us2);to2=fmaf(wz,s2-tv[2][t],to2);}
                    const float dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
                    vp01=pfma(pdup(wxy),ts01,vp01);vd01=pfma(pdup(wxy),to01,vd01);
                    g0=pfma(pdup(dxy),ts01,g0);g1=pfma(pdup(xdy),ts01,g1);g2=pfma(pdup(wxy),us01,g2);
                    vp[2]=fmaf(wxy,ts2,vp[2]);vd[2]=fmaf(wxy,to2,vd[2]);
                    G[6]=fmaf(dxy,ts2,G[6]);G[7]=fmaf(xdy,ts2,G[7]);G[8]=fmaf(wxy,us2,G[8]);}
                vp[0]=vp01.x;vp[1]=vp01.y;vd[0]=vd01.x;vd[1]=vd01.y;
                G[0]=g0.x;G[3]=g0.y;G[1]=g1.x;G[4]=g1.y;G[2]=g2.x;G[5]=g2.y;}
            else{
#pragma unroll
            for(int ox=0;ox<3;++ox)
#pragma unroll
            for(int oy=0;oy<3;++oy){
                T ts[3]={T(0),T(0),T(0)},us[3]={T(0),T(0),T(0)},to[3]={T(0),T(0),T(0)};
#pragma unroll
                for(int oz=0;oz<3;++oz){
                    const T wz=st.w[2][oz],dz=st.dw[2][oz];
                    const int t=tb+tile_addr(ox,oy,oz);
#pragma unroll
                    for(int a=0;a<3;++a){const T sa=tv[3+a][t];ts[a]+=wz*sa;us[a]+=dz*sa;to[a]+=wz*(sa-tv[a][t]);}}
                const T dxy=st.dw[0][ox]*st.w[1][oy],xdy=st.w[0][ox]*st.dw[1][oy],wxy=st.w[0][ox]*st.w[1][oy];
#pragma unroll
                for(int a=0;a<3;++a){
                    vp[a]+=wxy*ts[a];vd[a]+=wxy*to[a];
                    G[3*a]+=dxy*ts[a];G[3*a+1]+=xdy*ts[a];G[3*a+2]+=wxy*us[a];}}}
            T vf[3];
#pragma unroll
            for(int a=0;a<3;++a) vf[a]=V[a]+vd[a];
            const T dt=(T)(*S.dtp);
            if(sc.eos){
                // EOS fluid: density /= 1 + dt tr(grad v), Fe untouched (MPM_Example.cpp:646)
                const T rho=S.pcur[FJP*pc+i];
                S.pcur[FJP*pc+i]=rho/(T(1)+dt*(G[0]+G[4]+G[8]));}
            else{
                T GF[9];mat_mul(G,F,GF);
#pragma unroll
                for(int k=0;k<9;++k) S.pcur[(FF+k)*pc+i]=F[k]+dt*GF[k];}
            const T flip=sc.flip;
            bool inside=true,fin=true;
#pragma unroll
            for(int a=0;a<3;++a){
                const T vn=vf[a]*flip+vp[a]*(T(1)-flip);
                const T xn=X[a]+vp[a]*dt;
                S.pcur[(FV+a)*pc+i]=vn;S.pcur[(FX+a)*pc+i]=xn;
                if(!isfinite(xn)) fin=false;
                const T lo=T(0)+T(0.5)*sc.dx[a],hi=T(1)-T(0.5)*sc.dx[a];
                if(!(xn>=lo&&xn<=hi)) inside=false;}
            if(!fin){atomicOr(&S.ctr->error,ERR_NONFINITE);atomicMax(&S.ctr->bad_scene1,(unsigned)ci.scene+1u);}
            if(!inside) S.scn_cur[i]=-(ci.scene+1);
        }
        __syncthreads();
    }
}

// =====================================================================================
// K8: the substep size of mpm_advance_to_time (MPM_Driver::Advance_To_Target_Time,
// MPM_Driver.cpp:55-80). Per scene, max_v over its valid particles (Max_Particle_Velocity,
// MPM_Example.cpp:375-387) gives dt_s = clamp(cfl dx / max(max_v, 1e-2), dt_min, dt_max);
// the substep takes the smallest dt_s of the batch (one substep sequence for all scenes;
// with one scene this is the reference's rule). Then the end-of-frame split: the last
// substep lands exactly on the target, and the one before it halves the rest when less
// than two steps remain. The last CTA writes dt, advances the clock and sets `h_more`
// (when given) to whether another substep follows.
// =====================================================================================
template<class T> __global__ void __launch_bounds__(NODE_THREADS) k_cfl(DevState<T> S,FrameState* F,double* dt_out,unsigned long long h_more,int use_more)
{
    __shared__ SceneRed R;
    __shared__ unsigned long long dtbits;
    red_init(R,S.n_scenes);
    if(threadIdx.x==0) dtbits=dbits(F->dt_max);
    __syncthreads();
    const long long pc=S.pcap;
    for(long long i=blockIdx.x*(long long)blockDim.x+threadIdx.x;i<S.n_total;i+=(long long)gridDim.x*blockDim.x){
        const int s=S.scn_cur[i];
        if(s<0) continue;
        T a=T(0);
#pragma unroll
        for(int k=0;k<3;++k){const T v=S.pcur[(FV+k)*pc+i];a+=v*v;}
        const double v2=(double)a;
        if(v2>0.) atomicMax(&R.mx[s],dbits(v2));}
    const bool last=red_finish(R,S.n_scenes,S.acc2,&S.ctr->ticket[4],[&](int i,double,double mx,unsigned long long){
        const double vmax=sqrt(mx);
        const double dt=fmax(F->dt_min,fmin(F->dt_max,F->cfl*(double)S.scenes[i].dx[0]/fmax(vmax,1e-2)));
        atomicMin(&dtbits,dbits(dt));
    },false,true,false);
    if(last&&threadIdx.x==0){
        double dt=bitsd(dtbits);
        const double rem=F->target-F->time;
        int done=0;
        if(rem<dt*1.001){dt=rem;done=1;}
        else if(rem<2.*dt) dt=rem*0.5;
        F->substeps+=1;
        if(F->substeps>=F->max_substeps) done=1;
        F->time=(done&&dt==rem)?F->target:F->time+dt;
        F->dt_last=dt;F->done=done;
        *dt_out=dt;
        if(use_more) cudaGraphSetConditional((cudaGraphConditionalHandle)h_more,done?0u:1u);}
}
// Loop condition of the frame graph: continue while the latest substep did not end it.
static __global__ void k_frame_cond(const FrameState* F,unsigned long long h)
{
    if(threadIdx.x==0&&blockIdx.x==0) cudaGraphSetConditional((cudaGraphConditionalHandle)h,F->done?0u:1u);
}

} // namespace mpm
