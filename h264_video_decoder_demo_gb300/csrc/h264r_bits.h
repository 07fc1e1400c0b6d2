// h264r_bits.h — RBSP bit reading for the host-side syntax parser:
// emulation-prevention removal (7.4.1), fixed-length, Exp-Golomb (9.1) and
// more_rbsp_data (7.2).  Reads past the end return zeros and set `err`, so a
// truncated unit fails its range checks instead of reading out of bounds.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <vector>

namespace h264r {

// NAL unit payload (after the one-byte header) with every 0x000003 turned
// back into 0x0000.
inline void nal_to_rbsp(const uint8_t *p, size_t n, std::vector<uint8_t> &out)
{
    out.resize(n);
    uint8_t *o = out.data();
    size_t w = 0, i = 0;
    int zeros = 0;
    while (i < n) {
        if (zeros == 0) {
            // copy up to the next zero byte in one go
            const void *z = memchr(p + i, 0, n - i);
            const size_t end = z ? (size_t)((const uint8_t *)z - p) : n;
            memcpy(o + w, p + i, end - i);
            w += end - i;
            i = end;
            if (i == n) break;
        }
        const uint8_t b = p[i++];
        if (zeros >= 2 && b == 3) {
            zeros = 0;
            continue;
        }
        o[w++] = b;
        zeros = b == 0 ? zeros + 1 : 0;
    }
    out.resize(w);
}

// the 8 bytes of v in big-endian order, as a number
inline uint64_t be64(uint64_t v)
{
    const uint16_t probe = 1;
    uint8_t first;
    memcpy(&first, &probe, 1);
    return first ? __builtin_bswap64(v) : v;  // little-endian hosts swap
}

struct BitReader {
    const uint8_t *p = nullptr;
    size_t nbits = 0, pos = 0;
    size_t stop = 0;  // bit position of the rbsp_stop_one_bit
    bool err = false;

    BitReader() = default;
    BitReader(const uint8_t *data, size_t nbytes) { reset(data, nbytes); }

    void reset(const uint8_t *data, size_t nbytes)
    {
        p = data;
        nbits = nbytes * 8;
        pos = 0;
        err = false;
        // the last set bit of the unit is the stop bit (trailing zero bytes
        // of cabac_zero_words or padding are skipped)
        size_t n = nbytes;
        while (n > 0 && p[n - 1] == 0) n--;
        if (n == 0) {
            stop = 0;
        } else {
            int t = 0;
            while (!((p[n - 1] >> t) & 1)) t++;
            stop = n * 8 - 1 - t;
        }
    }

    // the 64 bits from the byte holding `pos`, big-endian (zeros past the end)
    uint64_t window() const
    {
        const size_t byte = pos >> 3, nbytes = nbits >> 3;
        uint64_t v = 0;
        if (byte + 8 <= nbytes) {
            memcpy(&v, p + byte, 8);
            v = be64(v);
        } else {
            for (int i = 0; i < 8; i++) v = (v << 8) | (byte + i < nbytes ? p[byte + i] : 0u);
        }
        return v;
    }

    // next k (1..32) bits without consuming them
    uint32_t peek(int k) const { return (uint32_t)((window() << (pos & 7)) >> (64 - k)); }

    // k (0..32) bits
    uint32_t u(int k)
    {
        if (k == 0) return 0;
        const uint32_t v = peek(k);
        pos += (size_t)k;
        if (pos > nbits) err = true;
        return v;
    }

    bool flag() { return u(1) != 0; }
    void skip(size_t k) { pos += k; if (pos > nbits) err = true; }

    uint32_t ue()
    {
        const uint32_t w = peek(32);
        if (w == 0) {  // more than 31 leading zeros: not a code of this decoder's range
            err = true;
            pos += 32;
            return 0;
        }
        const int lz = __builtin_clz(w);
        pos += (size_t)lz + 1;
        if (lz == 0) return pos > nbits ? (err = true, 0u) : 0u;
        const uint32_t v = ((1u << lz) - 1u) + u(lz);
        if (pos > nbits) err = true;
        return v;
    }

    int32_t se()
    {
        const uint32_t k = ue();
        return (k & 1) ? (int32_t)((k + 1) >> 1) : -(int32_t)(k >> 1);
    }

    // te(v) with range >= 1 (7.4.3 ref_idx when more than one reference)
    uint32_t te(int range) { return range > 1 ? ue() : (u(1) ^ 1u); }

    bool byte_aligned() const { return (pos & 7) == 0; }
    bool more_rbsp_data() const { return pos < stop; }
};

// RBSP bit writing for the seeded bitstream writer: fixed-length,
// Exp-Golomb (9.1) and trailing bits.  `buf` always holds every bit written
// so far, the last byte zero-padded, so a BitReader can read it back in place.
struct BitWriter {
    std::vector<uint8_t> buf;
    size_t nbits = 0;

    // k (0..32) bits of v, most significant first
    void u(int k, uint32_t v)
    {
        for (int i = k - 1; i >= 0; i--) {
            if ((nbits & 7) == 0) buf.push_back(0);
            if ((v >> i) & 1u) buf.back() |= (uint8_t)(0x80u >> (nbits & 7));
            nbits++;
        }
    }
    void flag(bool b) { u(1, b ? 1u : 0u); }
    void ue(uint32_t v)
    {
        const uint64_t k = (uint64_t)v + 1;
        int len = 0;
        while ((k >> len) > 1) len++;
        u(len, 0);
        // the code is len zeros, then k in len + 1 bits
        if (len >= 32) {
            u(1, 1);
            u(len, (uint32_t)(k & 0xFFFFFFFFu));
        } else {
            u(len + 1, (uint32_t)k);
        }
    }
    void se(int32_t v) { ue(v > 0 ? (uint32_t)(2 * (int64_t)v - 1) : (uint32_t)(-2 * (int64_t)v)); }
    // te(v) (7.4.3 ref_idx): one inverted bit when the range is 1
    void te(int range, uint32_t v)
    {
        if (range > 1) ue(v);
        else u(1, v ^ 1u);
    }
    bool byte_aligned() const { return (nbits & 7) == 0; }
    // rbsp_trailing_bits( ): the stop bit, then zeros to a byte boundary
    void trailing()
    {
        u(1, 1);
        while (!byte_aligned()) u(1, 0);
    }
};

// NAL unit in Annex B form: start code, header byte, payload with an
// emulation_prevention_three_byte after every two zero bytes that precede a
// byte <= 3 (7.4.1)
inline void put_nal(std::vector<uint8_t> &out, int nal_ref_idc, int nal_unit_type, const uint8_t *rbsp, size_t n)
{
    static const uint8_t start[4] = {0, 0, 0, 1};
    out.insert(out.end(), start, start + 4);
    out.push_back((uint8_t)(((nal_ref_idc & 3) << 5) | (nal_unit_type & 31)));
    int zeros = 0;
    for (size_t i = 0; i < n; i++) {
        if (zeros >= 2 && rbsp[i] <= 3) {
            out.push_back(3);
            zeros = 0;
        }
        out.push_back(rbsp[i]);
        zeros = rbsp[i] == 0 ? zeros + 1 : 0;
    }
}

}  // namespace h264r
