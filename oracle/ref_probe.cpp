// ref_probe.cpp — test infrastructure, never shipped: the reference's own
// CAVLC table decoders and CABAC tables exposed through a C interface, so
// that the parser's tables can be compared with them over every code word
// and every context
// (CH264ResidualBlockCavlc::coeff_token_table / get_total_zeros /
// get_run_before, H264ResidualBlockCavlc.cpp:580, 2087, 3023;
// CH264Golomb::get_me_golomb, H264Golomb.cpp:273).  Built by `make ref`
// into _ref/libref_probe.so from the reference's objects.
#include <cstdint>
#include <cstring>

#include "Bitstream.h"
#include "H264Golomb.h"
#include "H264ResidualBlockCavlc.h"
#include "H264Cabac.h"

namespace {

// bits consumed from a 4-byte buffer holding the 16-bit window then ones
int consumed(const CBitstream &bs, const uint8_t *buf)
{
    return (int)((bs.m_p - buf) * 8 + (8 - bs.m_bits_left));
}

}  // namespace

extern "C" int ref_probe_coeff_token(int nC, uint32_t window16, int out[3])
{
    CH264ResidualBlockCavlc c;
    int32_t len = 0, t1 = 0, tc = 0;
    if (c.coeff_token_table(nC, (uint16_t)window16, len, t1, tc) != 0) return -1;
    out[0] = len;
    out[1] = t1;
    out[2] = tc;
    return 0;
}

extern "C" int ref_probe_total_zeros(int max_coeff, int total_coeff, uint32_t window16, int out[2])
{
    uint8_t buf[4] = {(uint8_t)(window16 >> 8), (uint8_t)window16, 0xFF, 0xFF};
    CBitstream bs(buf, 4);
    CH264ResidualBlockCavlc c;
    int32_t z = 0;
    if (c.get_total_zeros(bs, max_coeff, total_coeff, z) != 0) return -1;
    out[0] = consumed(bs, buf);
    out[1] = z;
    return 0;
}

extern "C" int ref_probe_run_before(int zeros_left, uint32_t window16, int out[2])
{
    uint8_t buf[4] = {(uint8_t)(window16 >> 8), (uint8_t)window16, 0xFF, 0xFF};
    CBitstream bs(buf, 4);
    CH264ResidualBlockCavlc c;
    int32_t r = 0;
    if (c.get_run_before(bs, zeros_left, r) != 0) return -1;
    out[0] = consumed(bs, buf);
    out[1] = r;
    return 0;
}

// me(v) of codeNum, ChromaArrayType 1
extern "C" int ref_probe_cbp(uint32_t code_num, int intra)
{
    // ue(v) code word of code_num, left-aligned in 4 bytes
    const uint32_t v = code_num + 1;
    int n = 0;
    while ((v >> n) > 1) n++;
    const int len = 2 * n + 1;
    const uint32_t word = v << (32 - len);
    uint8_t buf[8] = {(uint8_t)(word >> 24), (uint8_t)(word >> 16), (uint8_t)(word >> 8), (uint8_t)word, 0xFF, 0xFF, 0xFF, 0xFF};
    CBitstream bs(buf, 8);
    CH264Golomb g;
    return g.get_me_golomb(bs, 1, intra ? Intra_4x4 : Inter);
}

// CABAC context initialisation values (m, n) of ctxIdx for a slice type
// (0 P, 1 B, 2 I) and cabac_init_idc (CH264Cabac::get_m_and_n,
// H264Cabac.cpp:36)
extern "C" int ref_probe_cabac_mn(int ctx_idx, int slice_type, int cabac_init_idc, int out[2])
{
    CH264Cabac c;
    int32_t m = 0, n = 0;
    if (c.get_m_and_n(ctx_idx, (H264_SLIECE_TYPE)slice_type, cabac_init_idc, m, n) != 0) return -1;
    out[0] = m;
    out[1] = n;
    return 0;
}

// one CABAC decision (CH264Cabac::DecodeDecision, H264Cabac.cpp:2577) from a
// given state, range and offset; the renormalisation reads zero bits.
// out: binVal, pStateIdx and valMPS after the decision, codIRange, codIOffset
extern "C" int ref_probe_cabac_decision(int p_state, int val_mps, int range, int offset, int out[5])
{
    uint8_t buf[16] = {0};
    CBitstream bs(buf, 16);
    CH264Cabac c;
    c.m_pStateIdxs[0] = p_state;
    c.m_valMPSs[0] = val_mps;
    c.m_codIRange = range;
    c.m_codIOffset = offset;
    int32_t bin = 0;
    if (c.DecodeDecision(bs, 0, bin) != 0) return -1;
    out[0] = bin;
    out[1] = c.m_pStateIdxs[0];
    out[2] = c.m_valMPSs[0];
    out[3] = c.m_codIRange;
    out[4] = c.m_codIOffset;
    return 0;
}
