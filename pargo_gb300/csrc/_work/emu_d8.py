import numpy as np, sys
sys.path.insert(0,'/root/repo')
from pargo_gb300 import synth
import oracle
f32=np.float32
K=f32(0.70710677); TLO=f32(0.99996948e-6); THI=f32(1.0000305e-6); M22=f32(2.0**-22); M20=f32(2.0**-20); M21=f32(2.0**-21); M48=f32(2.0**-48)
DIAG=[True,False,True,False,False,False,True,False,True]
W=[32,64,128,16,0,1,8,4,2]
def zd(z,i,j,f64):
    return f32(np.float64(z[i])-np.float64(z[j])) if f64 else f32(z[i]-z[j])
def cert(z, f64, dt=8):
    x=[None]*9; m=f32(-3e38); m2=f32(-3e38); k=0
    for i in range(9):
        if i==4: continue
        c=zd(z,4,i,f64); x[i]=f32(c*K) if DIAG[i] else c
        if x[i]>m: m2=m; m=x[i]; k=i
        else: m2=max(m2,x[i])
    if m<=0: return -1,'fast'
    em=f32(m*M22)
    if f32(m+em)<TLO: return -1,'fast'
    if not (f32(m-em)>THI): return None,'unsure'
    if f32(m-m2) > f32(THI + f32(f32(m+abs(m2))*M20)): return (k if dt==8 else W[k]),'fast'
    mask=1<<k
    for i in range(9):
        if i==4 or i==k: continue
        if DIAG[i]==DIAG[k]:
            g=zd(z,i,k,f64)
            if DIAG[k]: g=f32(g*K)
            err=f32(f32(abs(g)*M22)+f32(m*M48))
            if g<0 or (g>0 and g<=err): return None,'unsure'
        else:
            g=f32(m-x[i]); err=f32(f32(m+abs(x[i]))*M21)
            if g<=err: return None,'unsure'
        if f32(g+err)<TLO: mask|=1<<i
        elif not (f32(g-err)>THI): return None,'unsure'
    if dt==8:
        n=bin(mask).count('1')>>1
        idx=[i for i in range(9) if mask>>i&1]
        return idx[n],'ties'
    return sum(W[i] for i in range(9) if mask>>i&1),'ties'
O=oracle.Oracle()
def run(dem, f64, dt=8, n=40000, seed=0):
    ref=O.d8(dem,-9999.0,dir_type=dt)
    rng=np.random.default_rng(seed)
    R,C=dem.shape
    stats={'fast':0,'ties':0,'unsure':0}; bad=0
    rs=rng.integers(1,R-1,n); cs=rng.integers(1,C-1,n)
    for r,c in zip(rs,cs):
        win=dem[r-1:r+2,c-1:c+2].ravel()
        if (win==-9999).any(): continue
        code,kind=cert(win,f64,dt); stats[kind]+=1
        if code is not None and code!=ref[r,c]: bad+=1; print('MISMATCH',r,c,code,ref[r,c],win)
    print(stats,'bad',bad)
d=synth.hydro_dem(600,600,seed=1)
print('hydro f32'); run(d,False)
w=O.fill(d,-9999.0,gap=1e-3)
print('filled f64'); run(w,True)
print('filled f64 dir256'); run(w,True,256)
q=np.round(synth.fbm(300,300,5,0.7,0,50)).astype(np.float32)
print('quantised'); run(q,False)
print('quantised 256'); run(q,False,256)
wq=O.fill(q,-9999.0)
print('quantised filled'); run(wq,True)
