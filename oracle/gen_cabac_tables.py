"""Write h264_video_decoder_demo_gb300/csrc/h264r_cabac_init.inc: the CABAC
context initialisation values (m, n) of Tables 9-12 to 9-33 of the standard
for ctxIdx 0..459 (every context of 4:2:0 frame and MBAFF coding), for I
slices and for cabac_init_idc 0, 1 and 2.

No copy of the standard is available here, so the values are read once from
the reference decoder's own accessor (CH264Cabac::get_m_and_n,
H264Cabac.cpp:36) through oracle/_ref/libref_probe.so (`make -C oracle ref`)
and written in this repository's layout; tests/test_cabac.py compares the
committed table with the accessor over every entry.  Recipe, run where the
reference sources are present: python oracle/gen_cabac_tables.py
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "h264_video_decoder_demo_gb300", "csrc", "h264r_cabac_init.inc")
NCTX = 460


def main():
    lib = ctypes.CDLL(os.path.join(HERE, "_ref", "libref_probe.so"))
    out = (ctypes.c_int * 2)()
    rows = []
    # model 0: I slices; models 1..3: P / B slices with cabac_init_idc 0..2
    for model in range(4):
        st, idc = (2, 0) if model == 0 else (0, model - 1)
        vals = []
        for ctx in range(NCTX):
            rc = lib.ref_probe_cabac_mn(ctx, st, idc, out)
            vals.append((out[0], out[1]) if rc == 0 else (0, 0))
        rows.append(vals)
    with open(OUT, "w") as f:
        f.write("// Generated by oracle/gen_cabac_tables.py: CABAC (m, n) of Tables 9-12 to\n"
                "// 9-33, [model][ctxIdx], model 0 for I slices, 1 + cabac_init_idc otherwise.\n")
        f.write("static const int8_t kCabacInit[4][%d][2] = {\n" % NCTX)
        for vals in rows:
            f.write("    {\n")
            for i in range(0, NCTX, 8):
                f.write("        " + ", ".join("{%d, %d}" % v for v in vals[i:i + 8]) + ",\n")
            f.write("    },\n")
        f.write("};\n")
    print(OUT)


if __name__ == "__main__":
    main()
