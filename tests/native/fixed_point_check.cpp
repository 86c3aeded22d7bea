// Host check of the integer-only fixed-point conversions of fixed.cuh, which
// the kernels use for every energy / virial total and for the mixed path's
// per-atom sums.  The CUDA intrinsics the header calls are given host
// definitions here; atomicAdd and the shuffle are single-threaded stand-ins.
// Built and run by tests/test_fixed_point.py; prints "bad=0" when every
// conversion matches the correctly rounded reference.
#include <cstdint>
#include <cstring>
#include <cstdio>
#include <cmath>
#include <random>
static inline unsigned __float_as_uint(float x){unsigned u;memcpy(&u,&x,4);return u;}
static inline long long __double_as_longlong(double x){long long u;memcpy(&u,&x,8);return u;}
static inline double __longlong_as_double(long long u){double x;memcpy(&x,&u,8);return x;}
static inline int __clzll(long long v){return v==0?64:__builtin_clzll((unsigned long long)v);}
static inline unsigned long long atomicAdd(unsigned long long* p, unsigned long long v){auto o=*p;*p+=v;return o;}
static inline unsigned __shfl_xor_sync(unsigned, unsigned long long, int){return 0;}
#include "../../pysic_gb300/csrc/fixed.cuh"
using namespace pg;
int main(){
  std::mt19937_64 g(1); std::uniform_real_distribution<double> u(-1,1);
  long bad=0;
  // float -> fix -> double: compare with round(x*2^32)/2^32
  for(int t=0;t<2000000;++t){
    float x=(float)(u(g)*std::pow(10.0, (int)(g()%16)-8));
    long long f=fix_from_float(x);
    double ref=std::nearbyint((double)x*4294967296.0); // ties even vs away: only exact ties differ
    double xs=(double)x*4294967296.0; bool tie = std::fabs(xs-std::trunc(xs))==0.5;
    if (!tie && std::fabs((double)f-ref)>0.5) {if(bad++<5)printf("ff %g %lld %g\n",x,f,ref);}
    double d=fix_to_double(f);
    double r2=(double)f/4294967296.0;  // exact when |f|<2^53
    if (std::fabs((double)f)<9e15 && d!=r2){if(bad++<5)printf("fd %lld %.17g %.17g\n",f,d,r2);}
  }
  // double -> fix, large ints -> double rounding
  for(int t=0;t<2000000;++t){
    double x=u(g)*std::pow(10.0,(int)(g()%18)-10);
    long long f=fix_from_double(x);
    long double ref=std::nearbyintl((long double)x*4294967296.0L);
    long double xs2=(long double)x*4294967296.0L; bool tie2 = std::fabs(xs2-std::trunc(xs2))==0.5L;
    if (!tie2 && std::fabs((long double)f-ref)>0.5L){if(bad++<5)printf("df %.17g %lld\n",x,f);}
    long long v=(long long)(g()>>4); if(g()&1) v=-v;
    double d=fix_to_double(v);
    double r=(double)((long double)v/4294967296.0L);
    if (d!=r){if(bad++<5)printf("td %lld %.17g %.17g\n",v,d,r);}
  }
  // Fx128 from float/fix/double sums
  for(int t=0;t<200000;++t){
    Fx128 a=fx_zero(); long double s=0; long long fs=0; Fx128 b=fx_zero();
    for(int k=0;k<50;++k){ float x=(float)(u(g)*1000); a=fx_add(a,fx_from_float(x)); s+=x; long long f=fix_from_float(x); fs+=f; b=fx_add(b,fx_from_fix(f)); }
    double d=fx_to_double(a); if (std::fabs(d-(double)s)>1e-12*std::fabs((double)s)+1e-15){if(bad++<5)printf("fx %.17g %.17Lg\n",d,s);}
    double e=fx_to_double(b), e2=(double)((long double)fs/4294967296.0L); if (std::fabs(e-e2)>1e-12*std::fabs(e2)){if(bad++<5)printf("fxf %.17g %.17g\n",e,e2);}
    FxAcc acc{{0,0,0}}; Fx128 m=fx_from_double(-d); fx_red(&acc,a); fx_red(&acc,m); fx_red(&acc,b); fx_red(&acc,fx_neg(b));
    if (std::fabs(fx_to_double(fx_from_limbs(acc)))>1e-9){if(bad++<5)printf("limbs %.17g\n",fx_to_double(fx_from_limbs(acc)));}
    FxAcc acc2{{0,0,0}}; Fx128 ref=fx_zero();
    for(int k=0;k<40;++k){ Fx128 v=fx_from_double(u(g)*std::pow(10.0,(int)(g()%20)-6)); fx_red(&acc2,v); ref=fx_add(ref,v); }
    Fx128 got=fx_from_limbs(acc2); if(got.lo!=ref.lo||got.hi!=ref.hi){if(bad++<5)printf("limbsum mismatch\n");}
  }
  printf("nan: %g %g %g\n", fix_to_double(fix_from_float(NAN)), fx_to_double(fx_from_double(INFINITY)), fx_to_double(fx_from_float(-INFINITY)));
  printf("bad=%ld\n",bad);
}
