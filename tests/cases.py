"""Small tank configurations shared by the parity tests (sizes the CPU
oracle finishes in seconds)."""
from oracle.hos_oracle import default_input

# 2-D tank (n2 = 1), regular wave with a flap wavemaker
REG_1D = dict(inp=default_input(T_stop=30.0, amp_mono=0.025, nu_mono=1.0, toler=1e-7, f_out=10.0),
              n1=65, n2=1, n3=17, mHOS=3, p1=3, p2=1)
# higher order, p < M (partial dealiasing active at several orders)
REG_1D_M5 = dict(inp=default_input(T_stop=30.0, amp_mono=0.04, nu_mono=0.8, toler=1e-7, f_out=10.0),
                 n1=65, n2=1, n3=17, mHOS=5, p1=3, p2=1)
# 3-D tank, oblique regular wave (snake wavemaker)
REG_3D = dict(inp=default_input(T_stop=20.0, amp_mono=0.02, nu_mono=0.7, theta_mono=20.0, toler=1e-7,
                                f_out=4.0, ylen=20.0),
              n1=33, n2=17, n3=9, mHOS=3, p1=3, p2=3)
# sloshing (no wavemaker)
SLOSH = dict(inp=default_input(icase=1, islosh=3, aslosh=0.05, iabsnb=0, T_stop=5.0, toler=1e-8, f_out=2.0),
             n1=33, n2=1, n3=9, mHOS=4, p1=4, p2=1)
# JONSWAP with libgfortran random phases (icase 4), piston wavemaker
JONSWAP_1D = dict(inp=default_input(icase=4, Hs=0.05, Tp=1.2, gamma=3.3, iseed=513, igeom=1, T_stop=8.0,
                                    toler=1e-7, f_out=10.0),
                  n1=65, n2=1, n3=17, mHOS=3, p1=3, p2=1)

# 3-D tank with a long y axis: n2 - 1 = 128 takes the two-level y passes
# (free-surface grid and the phiadd_SL y sums); Nd2 - 1 = 257 is prime
WIDE_3D = dict(inp=default_input(T_stop=20.0, amp_mono=0.02, nu_mono=0.7, theta_mono=10.0, toler=1e-7,
                                 f_out=4.0, ylen=20.0),
               n1=17, n2=129, n3=9, mHOS=3, p1=3, p2=3)

# The reference's own Benchmark runs (configuration from their Ref_data input
# echo; fixtures tests/golden/ref_*.npz hold the reference's probe records)
REF_SLOSHING = dict(inp=default_input(xlen=50.0, ylen=29.74, h=5.0, icase=1, islosh=3, aslosh=0.2, iabsnb=0,
                                      T_stop=20.0, toler=1e-6, f_out=20.0, idim=1),
                    n1=129, n2=1, n3=33, mHOS=1, p1=1, p2=1)
REF_REGULAR_3D = dict(inp=default_input(xlen=46.4, ylen=29.74, h=5.0, icase=2, amp_mono=0.1, nu_mono=0.5588,
                                        theta_mono=30.0, ph_mono=0.0, ibat=3, xd_mono=25.0, i_wmk=1, igeom=2,
                                        d_hinge=2.147, iramp=1, Tramp=3.0, T_stop=40.0, iabsnb=1, xabsf=0.8,
                                        coeffabsf=1.0, toler=1e-4, f_out=10.0, idim=1),
                      n1=256, n2=32, n3=16, mHOS=3, p1=3, p2=3)
REF_IRREG_2D = dict(inp=default_input(xlen=120.0, ylen=100.0, h=5.0, icase=3, file_name="Hs4_Tp10", i_cut=0,
                                      ibat=2, i_wmk=2, igeom=2, d_hinge=1.0, iramp=0, Tramp=0.0, T_stop=50.0,
                                      iabsnb=1, xabsf=0.8, coeffabsf=1.0, toler=1e-4, f_out=30.0, idim=1),
                    n1=512, n2=1, n3=32, mHOS=3, p1=3, p2=1)


REF_IRREG_3D = dict(inp=default_input(xlen=46.4, ylen=29.74, h=5.0, icase=31, file_name="CAT1__22", i_cut=0,
                                      ibat=2, i_wmk=2, igeom=2, d_hinge=2.147, iramp=1, Tramp=3.0, T_stop=256.0,
                                      iabsnb=1, xabsf=0.8, coeffabsf=1.0, toler=1e-4, f_out=10.0, idim=1),
                    n1=256, n2=32, n3=16, mHOS=3, p1=3, p2=3)


def write_ref_txt(fx, directory, name="CAT1__22"):
    """The Edinburgh Designs .txt wave file of a reference fixture."""
    import os
    with open(os.path.join(directory, name + ".txt"), "w", encoding="latin-1") as f:
        for ln in fx["txt"]:
            f.write(str(ln) + "\n")


def write_ref_wave_files(fx, directory, name="Hs4_Tp10"):
    """The .cfg/.dat wave files of a reference fixture (the layout file2wave
    reads, wave_def.f90:181-278), rewritten with the stored values."""
    import os
    with open(os.path.join(directory, name + ".cfg"), "w") as f:
        for v in fx["cfg"]:
            f.write(f" {v} \n")
    with open(os.path.join(directory, name + ".dat"), "w") as f:
        for h, fr, a, an, ph in fx["components"]:
            f.write(f"{int(h)} , {float(fr)!r} , {float(a)!r} , {float(an)!r} , {float(ph)!r} ,\n")


# second-order wavemaker (i_wmk = 2), 2-D and 3-D
REG_1D_W2 = dict(inp=default_input(T_stop=30.0, amp_mono=0.03, nu_mono=0.8, toler=1e-7, f_out=10.0, i_wmk=2,
                                   iramp=1, Tramp=1.0),
                 n1=65, n2=1, n3=17, mHOS=3, p1=3, p2=1)
REG_3D_W2 = dict(inp=default_input(T_stop=20.0, amp_mono=0.02, nu_mono=0.7, theta_mono=20.0, toler=1e-7,
                                   f_out=4.0, ylen=20.0, i_wmk=2, iramp=1, Tramp=1.0),
                 n1=33, n2=17, n3=9, mHOS=3, p1=3, p2=3)

REG_1D_W3 = dict(REG_1D_W2, inp=dict(REG_1D_W2["inp"], i_wmk=3))
REG_3D_W3 = dict(REG_3D_W2, inp=dict(REG_3D_W2["inp"], i_wmk=3))

ALL = {"reg1d": REG_1D, "reg1d_w2": REG_1D_W2, "reg3d_w2": REG_3D_W2, "reg1d_w3": REG_1D_W3,
       "reg3d_w3": REG_3D_W3, "reg1d_m5": REG_1D_M5, "reg3d": REG_3D, "slosh": SLOSH, "jonswap1d": JONSWAP_1D,
       "wide3d": WIDE_3D}
