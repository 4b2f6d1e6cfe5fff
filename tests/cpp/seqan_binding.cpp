// Calls every overload of include/seqan_gb300_seqan.h with the SeqAn 2 types a caller uses
// (StringSet<Dna5String>, StringSet<Gaps<...>>, StringSet<Align<...>>, Score<int16_t|int, Simple>,
// Blosum62, AlignConfig, bands, Seed<Simple>, readRecord texts, BamAlignmentRecord) and prints
// every result in one canonical text form.
//
// Built two ways by tests/test_cpp_binding.py:
//   * default: the calls go to ExecutionPolicy<GB300, Vectorial>, i.e. through the C-ABI to the GPU;
//   * -DGBA_AS_REFERENCE: the same calls run by the reference itself -- the Sequential policy
//     (ExecutionPolicy<Serial, Serial>) for the set-versus-set overloads (the reference's scalar DP
//     pair by pair, the semantics the engine follows), the single-pair overloads in a loop where the reference has
//     no policy overload (one-versus-many, StringSet<Align>, extendSeed), the readRecord loop and
//     the per-record SAM / BAM writers.
// tests/golden/make_golden.py records the reference build's output as a fixture; the GPU test
// runs the default build and compares its output with it line by line.
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>

#include <seqan/align.h>
#include <seqan/align_parallel.h>
#include <seqan/bam_io.h>
#include <seqan/score.h>
#include <seqan/seeds.h>
#include <seqan/seq_io.h>

#ifndef GBA_AS_REFERENCE
#include "seqan_gb300_seqan.h"
#endif

using namespace seqan2;

#ifdef GBA_AS_REFERENCE
typedef Sequential TPolicy;   // ExecutionPolicy<Serial, Serial>: scalar, pair by pair
#else
typedef ExecutionPolicy<GB300, Vectorial> TPolicy;
#endif

template <typename TString>
static void print_scores(char const *name, TString const &s)
{
    std::cout << name << ':';
    for (size_t k = 0; k < length(s); ++k) std::cout << ' ' << int(s[k]);
    std::cout << '\n';
}

template <typename TGapsH, typename TGapsV>
static void print_pair(char const *name, size_t k, TGapsH &gh, TGapsV &gv)
{
    CharString cigar;
    getCigarString(cigar, gh, gv);
    std::cout << name << '[' << k << "]: " << gh << " | " << gv << " | " << clippedBeginPosition(gh) << ' '
              << clippedEndPosition(gh) << ' ' << clippedBeginPosition(gv) << ' ' << clippedEndPosition(gv) << " | "
              << cigar << '\n';
}

template <typename TSet>
static void print_gaps(char const *name, TSet &gapsH, TSet &gapsV)
{
    for (size_t k = 0; k < length(gapsH); ++k) print_pair(name, k, gapsH[k], gapsV[k]);
}

template <typename TAligns>
static void print_aligns(char const *name, TAligns &aligns)
{
    for (size_t k = 0; k < length(aligns); ++k) print_pair(name, k, row(aligns[k], 0), row(aligns[k], 1));
}

template <typename TSeeds>
static void print_seeds(char const *name, TSeeds const &seeds)
{
    for (size_t k = 0; k < length(seeds); ++k)
        std::cout << name << '[' << k << "]: " << beginPositionH(seeds[k]) << ' ' << endPositionH(seeds[k]) << ' '
                  << beginPositionV(seeds[k]) << ' ' << endPositionV(seeds[k]) << ' ' << lowerDiagonal(seeds[k]) << ' '
                  << upperDiagonal(seeds[k]) << '\n';
}

// Batch seed extension with the reference's seed and sequence types.
static void seeds_demo(TPolicy const &policy)
{
    StringSet<DnaString> dbs, qs;
    appendValue(dbs, "AACCCCTTTGGTGAAAAA");
    appendValue(qs, "AAACCCTTTGGGTTTTT");
    appendValue(dbs, "ttttcgatcgatgcttttt");
    appendValue(qs, "aaaacgatcgatgc");
    String<Seed<Simple>> seeds;
    appendValue(seeds, Seed<Simple>(4, 4, 3));
    appendValue(seeds, Seed<Simple>(4, 4, 9));
    String<Seed<Simple>> onShared;
    appendValue(onShared, Seed<Simple>(5, 5, 3));
    StringSet<String<AminoAcid>> pq;
    appendValue(pq, "CSNNHKMMMMAAGGW");
    String<AminoAcid> pdb = "CSNNHKMMMMAAGGW";
    Blosum62 b62(-9, -9);
#ifdef GBA_AS_REFERENCE
    (void)policy;
    for (size_t k = 0; k < length(seeds); ++k) {
        extendSeed(seeds[k], dbs[k], qs[k], EXTEND_BOTH, Score<int, Simple>(2, -1, -1), 1, GappedXDrop());
        extendSeed(seeds[k], dbs[k], qs[k], EXTEND_BOTH, Score<int, Simple>(0, -1, -1), 2, UnGappedXDrop());
        extendSeed(seeds[k], dbs[k], qs[k], EXTEND_LEFT, MatchExtend());
    }
    extendSeed(onShared[0], pdb, pq[0], EXTEND_BOTH, b62, 1, GappedXDrop());
#else
    extendSeed(policy, seeds, dbs, qs, EXTEND_BOTH, Score<int, Simple>(2, -1, -1), 1, GappedXDrop());
    extendSeed(policy, seeds, dbs, qs, EXTEND_BOTH, Score<int, Simple>(0, -1, -1), 2, UnGappedXDrop());
    extendSeed(policy, seeds, dbs, qs, EXTEND_LEFT, MatchExtend());
    extendSeed(policy, onShared, pdb, pq, EXTEND_BOTH, b62, 1, GappedXDrop());
#endif
    print_seeds("seeds", seeds);
    print_seeds("shared", onShared);
}

// FASTA / FASTQ input and SAM / BAM output.
static void io_demo(TPolicy const &policy)
{
    StringSet<CharString> ids, quals;
    StringSet<Dna5String> seqs;
    StringSet<String<AminoAcid>> prot;
    const std::string fa = ">r1 first\nACGT\nNN\n>r2\nacgt\n", pa = ">p\nMKV*\n", fq = "@q1\nACGT\n+\nIIII\n";
#ifdef GBA_AS_REFERENCE
    (void)policy;
    {
        std::istringstream s1(fa), s2(pa), s3(fq);
        auto i1 = directionIterator(s1, Input());
        auto i2 = directionIterator(s2, Input());
        auto i3 = directionIterator(s3, Input());
        CharString id, q;
        Dna5String seq;
        String<AminoAcid> pseq;
        while (!atEnd(i1)) { readRecord(id, seq, i1, Fasta()); appendValue(ids, id); appendValue(seqs, seq); }
        while (!atEnd(i2)) { readRecord(id, pseq, i2, Fasta()); appendValue(ids, id); appendValue(prot, pseq); }
        while (!atEnd(i3)) {
            readRecord(id, seq, q, i3, Fastq());
            appendValue(ids, id);
            appendValue(seqs, seq);
            appendValue(quals, q);
        }
    }
#else
    readRecords(policy, ids, seqs, fa, Fasta());
    readRecords(policy, ids, prot, pa, Fasta());
    readRecords(policy, ids, seqs, quals, fq, Fastq());
#endif
    for (size_t k = 0; k < length(ids); ++k) std::cout << "id[" << k << "]: " << ids[k] << '\n';
    for (size_t k = 0; k < length(seqs); ++k) std::cout << "seq[" << k << "]: " << seqs[k] << '\n';
    for (size_t k = 0; k < length(prot); ++k) std::cout << "prot[" << k << "]: " << prot[k] << '\n';
    for (size_t k = 0; k < length(quals); ++k) std::cout << "qual[" << k << "]: " << quals[k] << '\n';

    StringSet<CharString> names;
    appendValue(names, "chr1");
    appendValue(names, "chr2");
    NameStoreCache<StringSet<CharString>> cache(names);
    BamIOContext<StringSet<CharString>> context(names, cache);
    String<BamAlignmentRecord> records;
    for (int k = 0; k < 3; ++k) {
        BamAlignmentRecord r;
        r.qName = std::string("q") + std::to_string(k);
        r.flag = k == 2 ? 16 : 0;
        r.rID = k == 1 ? 1 : 0;
        r.beginPos = 10 + 100 * k;
        r.mapQ = 60 - k;
        appendValue(r.cigar, CigarElement<>('M', 4));
        if (k) appendValue(r.cigar, CigarElement<>('I', 1));
        r.rNextId = k == 0 ? BamAlignmentRecord::INVALID_REFID : 0;
        r.pNext = k == 0 ? BamAlignmentRecord::INVALID_POS : 500;
        r.tLen = k == 0 ? 0 : -300;
        r.seq = k ? "ACGTN" : "ACGT";
        r.qual = k == 1 ? "" : (k ? "IIIII" : "IIII");
        appendValue(records, r);
    }
    CharString sam, bam;
#ifdef GBA_AS_REFERENCE
    for (size_t k = 0; k < length(records); ++k) {
        write(sam, records[k], context, Sam());
        write(bam, records[k], context, Bam());
    }
#else
    write(policy, sam, records, context, Sam());
    write(policy, bam, records, context, Bam());
#endif
    std::cout << "sam:\n" << sam;
    std::cout << "bam:";
    for (size_t i = 0; i < length(bam); ++i)
        std::cout << std::hex << std::setw(2) << std::setfill('0') << (unsigned(bam[i]) & 0xffu);
    std::cout << std::dec << '\n';
}

int main()
{
    TPolicy policy;
    StringSet<Dna5String> setH, setV;
    appendValue(setH, "ACGTACGTTGACCA");
    appendValue(setH, "GATTACA");
    appendValue(setH, "TTGACCAGGTACGATNACCA");
    appendValue(setV, "ACGTTCGTTGCCA");
    appendValue(setV, "GATCACAA");
    appendValue(setV, "TTGACAGGTACGTTACCA");
    Score<int16_t, Simple> sc16(2, -4, -1, -6);
    Score<int, Simple> sc32(2, -3, -5, -5);

    print_scores("global16", globalAlignmentScore(policy, setH, setV, sc16));
    print_scores("global16_fe9", globalAlignmentScore(policy, setH, setV, sc16, AlignConfig<true, false, false, true>()));
    print_scores("global32_band", globalAlignmentScore(policy, setH, setV, sc32, -3, 3));
    print_scores("global32_fe15_band",
                 globalAlignmentScore(policy, setH, setV, sc32, AlignConfig<true, true, true, true>(), -3, 3));
    print_scores("local32", localAlignmentScore(policy, setH, setV, sc32));
    print_scores("local32_band", localAlignmentScore(policy, setH, setV, sc32, -2, 2));
#ifdef GBA_AS_REFERENCE
    {
        String<int16_t> e;
        for (size_t k = 0; k < length(setV); ++k) appendValue(e, globalAlignmentScore(setH[0], setV[k], sc16));
        print_scores("one_vs_many16", e);
    }
#else
    print_scores("one_vs_many16", globalAlignmentScore(policy, setH[0], setV, sc16));
#endif

    StringSet<String<AminoAcid>> pH, pV;
    appendValue(pH, "MKVLAAGIVGLLLA");
    appendValue(pH, "WWCHHKLMNPQ");
    appendValue(pV, "MKVIAAGLVGLA");
    appendValue(pV, "WCHHKIMNPPQ");
    Score<int16_t, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> blosum(-1, -11);
    print_scores("local_b62", localAlignmentScore(policy, pH, pV, blosum));
    print_scores("global_b62", globalAlignmentScore(policy, pH, pV, blosum));

    typedef Gaps<Dna5String> TGaps;
    StringSet<TGaps> gapsH, gapsV;
    for (size_t k = 0; k < length(setH); ++k) {
        appendValue(gapsH, TGaps(setH[k]));
        appendValue(gapsV, TGaps(setV[k]));
    }
    print_scores("gaps_global16", globalAlignment(policy, gapsH, gapsV, sc16));
    print_gaps("gaps_global16", gapsH, gapsV);
    print_scores("gaps_global16_fe6", globalAlignment(policy, gapsH, gapsV, sc16, AlignConfig<false, true, true, false>()));
    print_gaps("gaps_global16_fe6", gapsH, gapsV);
    print_scores("gaps_global32_band", globalAlignment(policy, gapsH, gapsV, sc32, -4, 4));
    print_gaps("gaps_global32_band", gapsH, gapsV);
    print_scores("gaps_local32", localAlignment(policy, gapsH, gapsV, sc32));
    print_gaps("gaps_local32", gapsH, gapsV);
    print_scores("gaps_local32_band", localAlignment(policy, gapsH, gapsV, sc32, -4, 4));
    print_gaps("gaps_local32_band", gapsH, gapsV);

    typedef Gaps<String<AminoAcid>> TPGaps;
    StringSet<TPGaps> pgH, pgV;
    for (size_t k = 0; k < length(pH); ++k) {
        appendValue(pgH, TPGaps(pH[k]));
        appendValue(pgV, TPGaps(pV[k]));
    }
    print_scores("gaps_local_b62", localAlignment(policy, pgH, pgV, blosum));
    print_gaps("gaps_local_b62", pgH, pgV);

    typedef Align<Dna5String> TAlign;
    StringSet<TAlign> aligns;
    for (size_t q = 0; q < length(setH); ++q) {
        TAlign al;
        resize(rows(al), 2);
        assignSource(row(al, 0), setH[q]);
        assignSource(row(al, 1), setV[q]);
        appendValue(aligns, al);
    }
#ifdef GBA_AS_REFERENCE
    {
        String<int16_t> n1;
        String<int> n2, n3, n4;
        for (size_t k = 0; k < length(aligns); ++k) appendValue(n1, globalAlignment(aligns[k], sc16));
        print_scores("align_global16", n1);
        print_aligns("align_global16", aligns);
        for (size_t k = 0; k < length(aligns); ++k)
            appendValue(n2, globalAlignment(aligns[k], sc32, AlignConfig<true, false, false, true>(), -3, 5));
        print_scores("align_global32_fe9_band", n2);
        print_aligns("align_global32_fe9_band", aligns);
        for (size_t k = 0; k < length(aligns); ++k) appendValue(n3, localAlignment(aligns[k], sc32));
        print_scores("align_local32", n3);
        print_aligns("align_local32", aligns);
        for (size_t k = 0; k < length(aligns); ++k) appendValue(n4, localAlignment(aligns[k], sc32, -2, 2));
        print_scores("align_local32_band", n4);
        print_aligns("align_local32_band", aligns);
    }
#else
    print_scores("align_global16", globalAlignment(policy, aligns, sc16));
    print_aligns("align_global16", aligns);
    print_scores("align_global32_fe9_band", globalAlignment(policy, aligns, sc32, AlignConfig<true, false, false, true>(), -3, 5));
    print_aligns("align_global32_fe9_band", aligns);
    print_scores("align_local32", localAlignment(policy, aligns, sc32));
    print_aligns("align_local32", aligns);
    print_scores("align_local32_band", localAlignment(policy, aligns, sc32, -2, 2));
    print_aligns("align_local32_band", aligns);
#endif
    seeds_demo(policy);
    io_demo(policy);
    return 0;
}
