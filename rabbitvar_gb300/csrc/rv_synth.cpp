// Native generator of seeded synthetic read sets for the large workloads
// (deep targeted panels, amplicon panels: tens of millions of reads).  It
// follows the model of rabbitvar_gb300/synth.py (simulate, amplicon_panel):
// Phred qualities from a mixture centred at 37, substitution errors with
// probability 10^(-q/10), N bases, soft clips, MAPQ 0 reads, planted SNVs /
// MNVs / indels carried with their allele fraction, oxidation-like C>A
// artifacts at a fixed quality, NM tags -- with its own random stream
// (xoshiro256**, seeded per region and sample), so its reads are not the
// numpy generator's reads.
//
// One call simulates the reads of one region and writes them, sorted by
// (position, fragment), in the GPU batch layout: fixed per-read fields at the
// caller's read offset, BAM-packed 4-bit bases and Phred qualities in 160-base
// slots, CIGAR words into a caller buffer (at most kMaxOps per read).  Calls
// for different regions are independent (the Python side runs them on a
// thread pool).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>

namespace {

constexpr int kMaxOps = 16;
constexpr int kStride = 160;  // bases per read slot (a multiple of 32)

struct Rng {
    uint64_t s[4];
    static uint64_t splitmix(uint64_t &x) {
        uint64_t z = (x += 0x9e3779b97f4a7c15ULL);
        z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
        z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
        return z ^ (z >> 31);
    }
    explicit Rng(uint64_t seed) {
        for (int i = 0; i < 4; i++) s[i] = splitmix(seed);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {  // xoshiro256** (Blackman and Vigna)
        const uint64_t r = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    int64_t integers(int64_t lo, int64_t hi) {  // [lo, hi)
        if (hi <= lo) return lo;
        return lo + (int64_t)(uniform() * (double)(hi - lo));
    }
    // Box-Muller: two standard normals per pair of uniforms (the second kept)
    bool have = false;
    double spare = 0.0;
    double normal(double mu, double sd) {
        if (have) {
            have = false;
            return mu + sd * spare;
        }
        double u1 = uniform(), u2 = uniform();
        if (u1 < 1e-300) u1 = 1e-300;
        const double r = std::sqrt(-2.0 * std::log(u1)), t = 6.283185307179586 * u2;
        spare = r * std::sin(t);
        have = true;
        return mu + sd * r * std::cos(t);
    }
};

const uint8_t kCode[4] = {1, 2, 4, 8};  // A C G T -> BAM 4-bit codes
constexpr uint8_t kCodeN = 15;

}  // namespace

extern "C" {

// One planted variant (0-based position of the first changed base).
typedef struct {
    int64_t pos;
    int32_t kind;       // 0 SNV, 1 MNV, 2 insertion, 3 deletion
    int32_t ref_len;    // deleted bases (deletion), changed bases (SNV/MNV)
    int32_t alt_off;    // alt bases (0..3 codes) in the alt buffer
    int32_t alt_len;
    double vaf;
    double strand_bias; // fraction of carriers forced onto `strand`
    int32_t strand;
    int32_t vq;         // > 0: quality forced on the changed bases of carriers
} rvs_variant;

typedef struct {
    uint64_t seed;
    int32_t read_len;
    int32_t amplicon;       // 1: fragments are the given amplicons (reads at both ends)
    double depth;
    int64_t lo, hi;         // span the fragments cover (0-based, half-open)
    double insert_mean, insert_sd;
    double softclip_frac, mapq0_frac, n_rate;
    double artifact_rate;   // C>A per C base
    int32_t artifact_q;     // quality of an artifact base (0: unchanged)
    int32_t tail_margin;
    int64_t name_base;
    double dup_frac;        // amplicon mode: exact duplicate pairs
} rvs_params;

// Number of reads rvs_simulate_region writes with these parameters: for
// random fragments 2 * round(depth * span / (2 * read_len)); in amplicon mode
// (which draws its duplicates first) 2 * (sum of amp_pairs + duplicates).
int64_t rvs_region_reads(const rvs_params *p, const int32_t *amp_pairs, int n_amp) {
    if (!p->amplicon) return 2 * (int64_t)std::llround(p->depth * (double)(p->hi - p->lo) / (2.0 * p->read_len));
    Rng rng(p->seed);
    int64_t n0 = 0;
    for (int k = 0; k < n_amp; k++) n0 += amp_pairs[k];
    int64_t d = 0;
    for (int64_t i = 0; i < n0; i++) d += rng.uniform() < p->dup_frac;
    return 2 * (n0 + d);
}

// Simulates one region; returns the number of CIGAR words written, or -1
// (bad read length, or n_expect differs from rvs_region_reads).  Outputs for
// its n reads: pos/mpos/isize/nm int32, flag uint16, mapq uint8, n_cigar
// uint16, name int64; seq (n * 80 bytes, packed) and qual (n * 160 bytes);
// cigar (at most n * kMaxOps words).
int64_t rvs_simulate_region(const uint8_t *genome, int64_t glen, const rvs_variant *vars, int n_vars,
                            const uint8_t *alt_buf, const rvs_params *p, const int64_t *amp_lo,
                            const int64_t *amp_hi, const int32_t *amp_pairs, int n_amp, int64_t n_expect,
                            int32_t *pos_out, int32_t *mpos_out, int32_t *isize_out, int32_t *nm_out,
                            uint16_t *flag_out, uint8_t *mapq_out, uint16_t *ncig_out, int64_t *name_out,
                            uint8_t *seq_out, uint8_t *qual_out, uint32_t *cigar_out) {
    const int L = p->read_len;
    if (L <= 0 || L > kStride) return -1;
    Rng rng(p->seed);
    double kErr[64];  // substitution probability 10^(-q/10) per quality
    for (int q = 0; q < 64; q++) kErr[q] = std::pow(10.0, -q / 10.0);
    // fragments: (start of read A, start of read B, insert)
    std::vector<int64_t> f_lo, f_hi;
    std::vector<int64_t> f_src;  // amplicon duplicates: the fragment they copy (-1: none)
    if (!p->amplicon) {
        const int64_t nf = std::llround(p->depth * (double)(p->hi - p->lo) / (2.0 * L));
        f_lo.resize(nf);
        f_hi.resize(nf);
        for (int64_t i = 0; i < nf; i++) {
            int64_t ins = std::llround(rng.normal(p->insert_mean, p->insert_sd));
            ins = std::max<int64_t>(L + 20, std::min<int64_t>(3 * L, ins));
            int64_t a = std::max<int64_t>(0, p->lo - L / 2);
            int64_t b = std::max<int64_t>(a + 1, p->hi - ins + L / 2);
            int64_t s = rng.integers(a, b);
            s = std::max<int64_t>(0, std::min<int64_t>(s, glen - p->tail_margin - ins));
            f_lo[i] = s;
            f_hi[i] = s + ins;
        }
        f_src.assign(nf, -1);
    } else {
        for (int k = 0; k < n_amp; k++)
            for (int j = 0; j < amp_pairs[k]; j++) {
                f_lo.push_back(amp_lo[k]);
                f_hi.push_back(amp_hi[k]);
            }
        const size_t n0 = f_lo.size();
        f_src.assign(n0, -1);
        for (size_t i = 0; i < n0; i++)
            if (rng.uniform() < p->dup_frac) {
                f_lo.push_back(f_lo[i]);
                f_hi.push_back(f_hi[i]);
                f_src.push_back((int64_t)i);
            }
    }
    const int64_t nf = (int64_t)f_lo.size();
    const int64_t n = 2 * nf;
    if (n != n_expect) return -1;
    // per read, in generation order; written out sorted
    std::vector<int32_t> pos(n), mpos(n), isize(n), nm(n);
    std::vector<uint16_t> flag(n), ncig(n);
    std::vector<uint8_t> mapq(n);
    std::vector<uint8_t> seq((size_t)n * kStride), qual((size_t)n * kStride);
    std::vector<uint32_t> cig((size_t)n * kMaxOps);
    std::vector<int64_t> frag(n);
    for (int64_t r = 0; r < n; r++) {
        const int64_t fi = r % nf;
        const bool b_read = r >= nf;
        const int64_t start = b_read ? f_hi[fi] - L : f_lo[fi];
        const bool rev = b_read;
        frag[r] = fi;
        uint8_t *sq = &seq[(size_t)r * kStride];
        uint8_t *ql = &qual[(size_t)r * kStride];
        // qualities: N(37, 2) declining by 3 along the sequencing direction,
        // 8 % of bases from U(2, 30), clipped to [2, 41]
        uint8_t qtmp[kStride];
        for (int i = 0; i < L; i++) {
            double q = rng.normal(37.0, 2.0) - 3.0 * i / (L - 1);
            if (rng.uniform() < 0.08) q = 2.0 + 28.0 * rng.uniform();
            q = std::rint(q);
            q = q < 2 ? 2 : (q > 41 ? 41 : q);
            qtmp[i] = (uint8_t)q;
        }
        for (int i = 0; i < L; i++) ql[i] = rev ? qtmp[L - 1 - i] : qtmp[i];
        // carried indels (at least 3 aligned bases on each side) and SNVs/MNVs
        int n_ind = 0;
        const rvs_variant *ind[8];
        uint8_t base[kStride];
        for (int i = 0; i < L; i++) base[i] = genome[start + i];
        bool carried_any_indel = false;
        for (int v = 0; v < n_vars; v++) {
            const rvs_variant &V = vars[v];
            const int vlen = std::max(V.ref_len, 1);
            if (V.pos + vlen <= start || V.pos >= start + L) continue;
            double pc = V.vaf;
            if (V.strand_bias > 0) {
                // a fraction strand_bias of carriers on the preferred strand (reads of
                // either strand are equally likely)
                pc = V.vaf * ((rev == (V.strand != 0)) ? 2.0 * V.strand_bias : 2.0 * (1.0 - V.strand_bias));
                pc = std::min(1.0, pc);
            }
            if (rng.uniform() >= pc) continue;
            if (V.kind <= 1) {
                for (int k = 0; k < V.alt_len; k++) {
                    int64_t col = V.pos + k - start;
                    if (col >= 0 && col < L) {
                        base[col] = alt_buf[V.alt_off + k];
                        if (V.vq > 0) ql[col] = (uint8_t)V.vq;
                    }
                }
            } else {
                int64_t off = V.pos - start;
                if (off >= 3 && off + V.ref_len <= L - 3 && start + L + V.ref_len + 4 < glen && n_ind < 8) {
                    ind[n_ind++] = &V;
                    carried_any_indel = true;
                }
            }
        }
        int nops = 0;
        uint32_t *cg = &cig[(size_t)r * kMaxOps];
        int64_t read_pos = start;
        if (carried_any_indel) {
            // rebuild bases and CIGAR from the haplotype (SNVs kept on matched bases)
            for (int a = 1; a < n_ind; a++)  // by position (at most 8)
                for (int b = a; b > 0 && ind[b]->pos < ind[b - 1]->pos; b--) std::swap(ind[b], ind[b - 1]);
            uint8_t nb[kStride];
            int nbn = 0, j = 0;
            int64_t gp = start;
            auto push = [&](int op, int ln) {
                if (ln <= 0) return;
                if (nops > 0 && (int)(cg[nops - 1] & 15u) == op) cg[nops - 1] += (uint32_t)ln << 4;
                else if (nops < kMaxOps) cg[nops++] = ((uint32_t)ln << 4) | (uint32_t)op;
            };
            while (nbn < L) {
                if (j < n_ind && gp == ind[j]->pos) {
                    const rvs_variant &V = *ind[j++];
                    if (V.kind == 2) {
                        int k = std::min(V.alt_len, L - nbn);
                        for (int t = 0; t < k; t++) nb[nbn++] = alt_buf[V.alt_off + t];
                        push(1, k);
                    } else {
                        push(2, V.ref_len);
                        gp += V.ref_len;
                    }
                    continue;
                }
                const int64_t col = gp - start;
                nb[nbn++] = (col >= 0 && col < L) ? base[col] : genome[gp];
                push(0, 1);
                gp++;
            }
            if (nops > 0 && (cg[nops - 1] & 15u) == 1u) cg[nops - 1] = (cg[nops - 1] & ~15u) | 4u;
            memcpy(base, nb, (size_t)L);
        }
        // artifacts, errors, N bases -> 4-bit codes
        uint8_t code[kStride];
        for (int i = 0; i < L; i++) {
            uint8_t b = base[i];
            const double perr = kErr[ql[i] & 63];
            if (p->artifact_rate > 0 && b == 1 && rng.uniform() < p->artifact_rate) {
                b = 0;
                if (p->artifact_q > 0) ql[i] = (uint8_t)p->artifact_q;
            }
            if (rng.uniform() < perr) b = (uint8_t)((b + rng.integers(1, 4)) % 4);
            code[i] = kCode[b];
            if (rng.uniform() < p->n_rate) {
                code[i] = kCodeN;
                ql[i] = 2;
            }
        }
        mapq[r] = rng.uniform() < p->mapq0_frac ? 0 : 60;
        // soft clips on reads without indels
        if (!carried_any_indel && rng.uniform() < p->softclip_frac) {
            const int k = (int)rng.integers(5, 31);
            const bool five = rng.uniform() < 0.5;
            const bool junk = rng.uniform() < 0.5;
            if (junk)
                for (int t = 0; t < k; t++) code[five ? t : L - k + t] = kCode[rng.integers(0, 4)];
            if (five) {
                cg[0] = ((uint32_t)k << 4) | 4u;
                cg[1] = ((uint32_t)(L - k) << 4) | 0u;
                read_pos = start + k;
            } else {
                cg[0] = ((uint32_t)(L - k) << 4) | 0u;
                cg[1] = ((uint32_t)k << 4) | 4u;
            }
            nops = 2;
        }
        if (nops == 0) {
            cg[0] = ((uint32_t)L << 4) | 0u;
            nops = 1;
        }
        ncig[r] = (uint16_t)nops;
        // NM over the alignment
        int m = 0, q = 0;
        int64_t rp = read_pos;
        for (int k = 0; k < nops; k++) {
            const int op = (int)(cg[k] & 15u), ln = (int)(cg[k] >> 4);
            if (op == 0) {
                for (int t = 0; t < ln; t++) m += code[q + t] != kCode[genome[rp + t]];
                q += ln;
                rp += ln;
            } else if (op == 1) {
                m += ln;
                q += ln;
            } else if (op == 2) {
                m += ln;
                rp += ln;
            } else if (op == 4) {
                q += ln;
            }
        }
        nm[r] = m;
        for (int i = 0; i < L; i++) sq[i] = code[i];
        pos[r] = (int32_t)read_pos;
        isize[r] = (int32_t)(b_read ? -(f_hi[fi] - f_lo[fi]) : (f_hi[fi] - f_lo[fi]));
        flag[r] = (uint16_t)(1 | 2 | (rev ? 16 : 0) | (rev ? 0 : 32) | (b_read ? 128 : 64));
    }
    // amplicon duplicates: exact copies of their original pair's two reads
    for (int64_t dst = 0; dst < nf; dst++) {
        const int64_t src = f_src[dst];
        if (src < 0) continue;
        for (int half = 0; half < 2; half++) {
            const int64_t a = src + half * nf, b = dst + half * nf;
            memcpy(&seq[(size_t)b * kStride], &seq[(size_t)a * kStride], kStride);
            memcpy(&qual[(size_t)b * kStride], &qual[(size_t)a * kStride], kStride);
            memcpy(&cig[(size_t)b * kMaxOps], &cig[(size_t)a * kMaxOps], kMaxOps * 4);
            ncig[b] = ncig[a];
            nm[b] = nm[a];
            mapq[b] = mapq[a];
            pos[b] = pos[a];
        }
    }
    // mate fields follow the (possibly clipped) alignment starts
    for (int64_t r = 0; r < n; r++) mpos[r] = pos[r < nf ? r + nf : r - nf];
    // sort by (position, fragment)
    std::vector<int64_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        return pos[a] != pos[b] ? pos[a] < pos[b] : frag[a] < frag[b];
    });
    int64_t nw = 0;
    for (int64_t i = 0; i < n; i++) {
        const int64_t r = order[i];
        pos_out[i] = pos[r];
        mpos_out[i] = mpos[r];
        isize_out[i] = isize[r];
        nm_out[i] = nm[r];
        flag_out[i] = flag[r];
        mapq_out[i] = mapq[r];
        ncig_out[i] = ncig[r];
        name_out[i] = p->name_base + frag[r];
        uint8_t *so = seq_out + (size_t)i * (kStride / 2);
        const uint8_t *si = &seq[(size_t)r * kStride];
        for (int t = 0; t < kStride / 2; t++) so[t] = (uint8_t)((si[2 * t] << 4) | si[2 * t + 1]);
        memcpy(qual_out + (size_t)i * kStride, &qual[(size_t)r * kStride], kStride);
        for (int k = 0; k < ncig[r]; k++) cigar_out[nw++] = cig[(size_t)r * kMaxOps + k];
    }
    return nw;
}

int rvs_max_ops(void) { return kMaxOps; }

}  // extern "C"
