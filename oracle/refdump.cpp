// Oracle test infrastructure: harness linked against the UNMODIFIED
// reference objects (built by oracle/Makefile into oracle/_ref/).  It runs
// the reference's per-region pipeline exactly as one_region_run does
// (src/modes/simpleMode.cpp:18-64) and prints, sorted, the maps at three
// boundaries:
//   stage P  after CigarParser::process        (src/parseCigar.cpp:410-440)
//   stage R  after VariationRealigner::process (src/VariationRealigner.cpp:135-161)
//   stage V  after ToVarsBuilder::process      (src/ToVarsBuilder.cpp:97-205)
// The printed dump is the golden record the project's CPU restatement and the
// GPU path are compared against.
//
// usage: rvref_dump -G ref.fa -b in.bam -R chr:start-end [-k 0|1] [-f F]
//                   [-u] [-t] [-q Q] [-X N] [-m N] [-Q N] [-F hex] [-T N] [-M N] [-3]
//                   [-O F] [-P N] [-o F] [-B N] [-x N] [-r N] [-V F] [-Y N] [--UN] [-stage PRV]
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <algorithm>
#include <string>
#include <vector>

#include "Configuration.h"
#include "Region.h"
#include "recordPreprocessor.h"
#include "parseCigar.h"
#include "VariationRealigner.h"
#include "ToVarsBuilder.h"
#include "scopedata/InitialData.h"
#include "data/data_pool.h"

static void pvar(const char *tag, int pos, const std::string &key, const Variation *v) {
    printf("%s\t%d\t%s\t%d\t%d\t%d\t%.17g\t%.17g\t%.17g\t%.17g\t%d\t%d\t%d\t%d\t%d\t%.17g\t%d\n", tag, pos,
           key.c_str(), v->varsCount, v->varsCountOnForward, v->varsCountOnReverse, v->meanPosition,
           v->meanQuality, v->meanMappingQuality, v->numberOfMismatches, v->lowQualityReadsCount,
           v->highQualityReadsCount, (int)v->pstd, (int)v->qstd, v->pp, v->pq, v->extracnt);
}

template <class M>
static std::vector<int> sorted_keys(const M &m) {
    std::vector<int> k;
    for (auto &e : m) k.push_back(e.first);
    std::sort(k.begin(), k.end());
    return k;
}

static void dump_varmap(const char *tag, robin_hood::unordered_map<int, VariationMap *> *m) {
    for (int p : sorted_keys(*m)) {
        auto &vm = m->at(p)->variation_map;
        std::vector<std::string> ks;
        for (auto &e : vm) ks.push_back(e.first);
        std::sort(ks.begin(), ks.end());
        for (auto &k : ks) pvar(tag, p, k, vm.at(k));
    }
}

static void dump_sclips(const char *tag, robin_hood::unordered_map<int, Sclip *> *m) {
    for (int p : sorted_keys(*m)) {
        Sclip *s = m->at(p);
        pvar(tag, p, "*", s);
        for (auto &ent : s->nt) {
            std::vector<char> cs;
            for (auto &c : ent.second) cs.push_back(c.first);
            std::sort(cs.begin(), cs.end());
            for (char c : cs) {
                char key[64];
                snprintf(key, sizeof key, "%d:%c:%d", ent.first, c, ent.second.at(c));
                auto sit = s->seq.find(ent.first);
                const Variation *sv = nullptr;
                if (sit != s->seq.end()) {
                    auto it2 = sit->second.find(c);
                    if (it2 != sit->second.end()) sv = it2->second;
                }
                if (sv) pvar(tag, p, key, sv);
                else printf("%s\t%d\t%s\tmissing\n", tag, p, key);
            }
        }
    }
}

static void dump_counts(const char *tag,
                        robin_hood::unordered_map<int, robin_hood::unordered_map<string, int>> *m) {
    for (int p : sorted_keys(*m)) {
        auto &vm = m->at(p);
        std::vector<std::string> ks;
        for (auto &e : vm) ks.push_back(e.first);
        std::sort(ks.begin(), ks.end());
        for (auto &k : ks) printf("%s\t%d\t%s\t%d\n", tag, p, k.c_str(), vm.at(k));
    }
}

static void dump_cov(const char *tag, robin_hood::unordered_map<int, int> *m) {
    for (int p : sorted_keys(*m)) printf("%s\t%d\t%d\n", tag, p, m->at(p));
}

static void dump_variant(int pos, const char *kind, const Variant *v) {
    printf("V\t%d\t%s\t%s\t%d\t%d\t%d\t%s\t%.17g\t%.17g\t%d\t%.17g\t%d\t%.17g\t%.17g\t%.17g\t%.17g"
           "\t%d\t%.17g\t%d\t%.17g\t%d\t%d\t%s\t%s\t%d\t%d\t%d\t%d\t%d\t%s\t%s\t%s\n",
           pos, kind, v->descriptionString.c_str(), v->positionCoverage, v->varsCountOnForward,
           v->varsCountOnReverse, v->strandBiasFlag.c_str(), v->frequency, v->meanPosition,
           (int)v->isAtLeastAt2Positions, v->meanQuality, (int)v->hasAtLeast2DiffQualities,
           v->meanMappingQuality, v->highQualityToLowQualityRatio, v->highQualityReadsFrequency,
           v->extraFrequency, v->shift3, v->msi, v->msint, v->numberOfMismatches, v->hicnt, v->hicov,
           v->leftseq.c_str(), v->rightseq.c_str(), v->startPosition, v->endPosition,
           v->refForwardCoverage, v->refReverseCoverage, v->totalPosCoverage, v->genotype.c_str(),
           v->refallele.c_str(), v->varallele.c_str());
}

int main(int argc, char **argv) {
    Configuration *conf = new Configuration();
    conf->patterns = new Patterns();
    std::string region_s, stages = "PRV";
    conf->threads = 1;
    conf->fisher = false;
    for (int i = 1; i < argc; ++i) {
        std::string a = argv[i];
        auto nxt = [&]() { return std::string(argv[++i]); };
        if (a == "-G") conf->fasta = nxt();
        else if (a == "-b") conf->bam = BamNames(nxt());
        else if (a == "-R") region_s = nxt();
        else if (a == "-k") conf->performLocalRealignment = (nxt() == "1");
        else if (a == "-f") conf->freq = atof(nxt().c_str());
        else if (a == "-u") conf->uniqueModeAlignmentEnabled = true;
        else if (a == "-t") conf->removeDuplicatedReads = true;
        else if (a == "-q") conf->goodq = atof(nxt().c_str());
        else if (a == "-X") conf->vext = atoi(nxt().c_str());
        else if (a == "-m") conf->mismatch = atoi(nxt().c_str());
        else if (a == "-Q") conf->mappingQuality = atoi(nxt().c_str());
        else if (a == "-F") conf->samfilter = nxt();
        // the other options the path reads, set as Launcher.cpp:388-470 sets them
        else if (a == "-T") conf->trimBasesAfter = atoi(nxt().c_str());
        else if (a == "-M") conf->minmatch = atoi(nxt().c_str());
        else if (a == "-3") conf->moveIndelsTo3 = true;
        else if (a == "-O") conf->mapq = atof(nxt().c_str());
        else if (a == "-P") conf->readPosFilter = atoi(nxt().c_str());
        else if (a == "-o") conf->qratio = atof(nxt().c_str());
        else if (a == "-B") conf->minBiasReads = atoi(nxt().c_str());
        else if (a == "-x") conf->numberNucleotideToExtend = atoi(nxt().c_str());
        else if (a == "-r") conf->minr = atoi(nxt().c_str());
        else if (a == "-V") conf->lofreq = atof(nxt().c_str());
        else if (a == "-Y") conf->referenceExtension = atoi(nxt().c_str());
        else if (a == "--UN") conf->uniqueModeSecondInPairEnabled = true;
        else if (a == "-stage") stages = nxt();
        else { fprintf(stderr, "unknown arg %s\n", a.c_str()); return 2; }
    }
    size_t colon = region_s.rfind(':');
    size_t dash = region_s.find('-', colon);
    // -x widens the -R region on both sides (RegionBuilder.cpp:187-188)
    int r_start = atoi(region_s.substr(colon + 1, dash - colon - 1).c_str()) - conf->numberNucleotideToExtend;
    int r_end = atoi(region_s.substr(dash + 1).c_str()) + conf->numberNucleotideToExtend;
    if (r_start > r_end) r_start = r_end;
    Region region(region_s.substr(0, colon), r_start, r_end, "g");

    std::vector<bamReader> readers;
    for (const std::string &bn : ssplit(conf->bam.getBam1(), ":")) {
        samFile *in = sam_open(bn.c_str(), "r");
        if (!in) { fprintf(stderr, "cannot open %s\n", bn.c_str()); return 1; }
        bam_hdr_t *h = sam_hdr_read(in);
        hts_idx_t *idx = sam_index_load(in, bn.c_str());
        for (int t = 0; t < h->n_targets; ++t) conf->chrLengths[h->target_name[t]] = h->target_len[t];
        readers.emplace_back(in, h, idx);
    }
    dataPool pool(region.end - region.start);
    pool.reset();
    InitialData *init = new InitialData;
    RecordPreprocessor *pre = new RecordPreprocessor(region, conf, readers);
    pre->makeReference(conf->fasta);
    std::set<std::string> splice;
    Scope<InitialData> initialScope(conf->bam.getBam1(), region, &pre->reference, 0, &splice, readers, init);
    CigarParser cp(pre, &pool);
    Scope<VariationData> svd = cp.process(initialScope);
    if (stages.find('P') != std::string::npos) {
        VariationData *d = svd.data;
        printf("P_ML\t%d\n", svd.maxReadLength);
        dump_varmap("PN", d->nonInsertionVariants);
        dump_varmap("PI", d->insertionVariants);
        dump_cov("PC", d->refCoverage);
        dump_sclips("PS5", d->softClips5End);
        dump_sclips("PS3", d->softClips3End);
        dump_counts("PCI", d->positionToInsertionCount);
        dump_counts("PCD", d->positionToDeletionCount);
        dump_counts("PMN", d->mnp);
    }
    VariationRealigner vr(conf, &pool);
    Scope<RealignedVariationData> rvd = vr.process(svd);
    if (stages.find('R') != std::string::npos) {
        RealignedVariationData *d = rvd.data;
        dump_varmap("RN", d->nonInsertionVariants);
        dump_varmap("RI", d->insertionVariants);
        dump_cov("RC", d->refCoverage);
    }
    ToVarsBuilder tb(conf);
    Scope<AlignedVarsData> *avd = tb.process(rvd);
    if (stages.find('V') != std::string::npos) {
        auto &av = avd->data->alignedVariants;
        for (int p : sorted_keys(av)) {
            Vars *vs = av.at(p);
            if (vs->referenceVariant) dump_variant(p, "ref", vs->referenceVariant);
            for (Variant *v : vs->variants) dump_variant(p, "var", v);
        }
    }
    return 0;
}
