"""FP32 against the FP64 build of the same kernels on the dam break
(dp = 0.002 m, 49,833 particles, mDBC, c0 = 35 m/s) over 1.0 s of physical
time: particle-position differences, water front (largest fluid x below
5 cm) and the water level at the four gauges of
cases/damBreakLong_mDBC/constants.h, every 0.05 s.  A measurement script,
not a test (the FP64 build takes ~7 minutes on a GB300):

    python tests/precision_study.py
"""
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
from tinysph_old_gb300 import cases, sph  # noqa: E402

def main():
    case = cases.dam_break_benchmark(0.002)
    print('dam break 0.002 np', case.np, 'dt', case.dt)
    nst = int(round(1.0/case.dt))
    sa = sph.ParticleSystem.from_case(case,'fp32'); sb = sph.ParticleSystem.from_case(case,'fp64')
    every = int(round(0.05/case.dt))
    done=0; ta=tb=0
    gx = np.array([0.3,0.865,1.114,1.3625])
    while done < nst:
        t0=time.time(); sa.step(0, case.dt, every); sa.sync(); ta+=time.time()-t0
        t0=time.time(); sb.step(0, case.dt, every); sb.sync(); tb+=time.time()-t0
        done+=every
        a=sa.download(); b=sb.download()
        same = np.array_equal(a['index'], b['index'])
        fa, fb = sa.water_front(0.05), sb.water_front(0.05)
        wa, wb = sa.water_level(gx, 0.0), sb.water_level(gx, 0.0)
        if same:
            fl=a['type']==0
            d=np.linalg.norm(a['r'][fl]-b['r'][fl],axis=1)
            print('t %.2f'%(done*case.dt), 'np', len(a['index']), 'pos err mean %.2e p99 %.2e max %.2e'%(d.mean(), np.percentile(d,99), d.max()), 'front %.5f %.5f rel %.2e'%(fa, fb, abs(fa-fb)/fb), 'wl', np.round(wa,4), np.round(wb,4))
        else:
            print('t %.2f'%(done*case.dt), 'particle sets differ', len(a['index']), len(b['index']), 'front %.5f %.5f'%(fa, fb), 'wl', np.round(wa,4), np.round(wb,4))
    print('times fp32 %.1f s fp64 %.1f s for %d steps'%(ta, tb, done))


if __name__ == "__main__":
    main()
