// Instantiates every overload of include/seqan_gb300_seqan.h with the SeqAn 2 types a caller
// uses (StringSet<Dna5String>, StringSet<Gaps<...>>, Score<int16_t|int, Simple>, Blosum62,
// AlignConfig, bands).  Built by tests/test_cpp_binding.py against the reference's headers and
// linked against libseqan_gb300.so; with a GPU it prints each result for comparison with the
// same calls under ExecutionPolicy<Parallel, Vectorial>.
#include <iostream>

#include <seqan/align.h>
#include <seqan/align_parallel.h>
#include <seqan/score.h>

#include "seqan_gb300_seqan.h"

using namespace seqan2;

// Batch seed extension with the reference's seed and sequence types.
static void seeds_demo(ExecutionPolicy<GB300, Vectorial> const &gpu)
{
    StringSet<DnaString> dbs, qs;
    appendValue(dbs, "AACCCCTTTGGTGAAAAA");
    appendValue(qs, "AAACCCTTTGGGTTTTT");
    appendValue(dbs, "ttttcgatcgatgcttttt");
    appendValue(qs, "aaaacgatcgatgc");
    String<Seed<Simple>> seeds;
    appendValue(seeds, Seed<Simple>(4, 4, 3));
    appendValue(seeds, Seed<Simple>(4, 4, 9));
    extendSeed(gpu, seeds, dbs, qs, EXTEND_BOTH, Score<int, Simple>(2, -1, -1), 1, GappedXDrop());
    extendSeed(gpu, seeds, dbs, qs, EXTEND_BOTH, Score<int, Simple>(0, -1, -1), 2, UnGappedXDrop());
    extendSeed(gpu, seeds, dbs, qs, EXTEND_LEFT, MatchExtend());
    String<Seed<Simple>> onShared;
    appendValue(onShared, Seed<Simple>(5, 5, 3));
    StringSet<String<AminoAcid>> pq;
    appendValue(pq, "CSNNHKMMMMAAGGW");
    String<AminoAcid> pdb = "CSNNHKMMMMAAGGW";
    Blosum62 b62(-9, -9);
    extendSeed(gpu, onShared, pdb, pq, EXTEND_BOTH, b62, 1, GappedXDrop());
    for (size_t k = 0; k < length(seeds); ++k)
        std::cout << beginPositionH(seeds[k]) << " " << endPositionH(seeds[k]) << "\n";
    std::cout << beginPositionH(onShared[0]) << " " << endPositionH(onShared[0]) << "\n";
}

// FASTA / FASTQ input and SAM / BAM output through the GB300 overloads.
static void io_demo(ExecutionPolicy<GB300, Vectorial> const &gpu)
{
    StringSet<CharString> ids, quals;
    StringSet<Dna5String> seqs;
    readRecords(gpu, ids, seqs, std::string(">r1 first\nACGT\nNN\n>r2\nacgt\n"), Fasta());
    StringSet<String<AminoAcid>> prot;
    readRecords(gpu, ids, prot, std::string(">p\nMKV*\n"), Fasta());
    readRecords(gpu, ids, seqs, quals, std::string("@q1\nACGT\n+\nIIII\n"), Fastq());
    StringSet<CharString> names;
    appendValue(names, "chr1");
    NameStoreCache<StringSet<CharString>> cache(names);
    BamIOContext<StringSet<CharString>> context(names, cache);
    String<BamAlignmentRecord> records;
    BamAlignmentRecord r;
    r.qName = "q1";
    r.rID = 0;
    r.beginPos = 10;
    appendValue(r.cigar, CigarElement<>('M', 4));
    r.seq = "ACGT";
    r.qual = "IIII";
    appendValue(records, r);
    CharString sam, bam;
    write(gpu, sam, records, context, Sam());
    write(gpu, bam, records, context, Bam());
    std::cout << length(ids) << ' ' << length(seqs) << ' ' << length(sam) << ' ' << length(bam) << '\n';
}

int main()
{
    ExecutionPolicy<GB300, Vectorial> gpu;
    StringSet<Dna5String> setH, setV;
    appendValue(setH, "ACGTACGTTGACCA");
    appendValue(setH, "GATTACA");
    appendValue(setV, "ACGTTCGTTGCCA");
    appendValue(setV, "GATCACAA");
    Score<int16_t, Simple> sc16(2, -4, -1, -6);
    Score<int, Simple> sc32(2, -3, -5, -5);

    String<int16_t> a = globalAlignmentScore(gpu, setH, setV, sc16);
    String<int16_t> b = globalAlignmentScore(gpu, setH, setV, sc16, AlignConfig<true, false, false, true>());
    String<int> c = globalAlignmentScore(gpu, setH, setV, sc32, -3, 3);
    String<int> d = globalAlignmentScore(gpu, setH, setV, sc32, AlignConfig<true, true, true, true>(), -3, 3);
    String<int16_t> e = globalAlignmentScore(gpu, setH[0], setV, sc16);
    String<int> f = localAlignmentScore(gpu, setH, setV, sc32);
    String<int> g = localAlignmentScore(gpu, setH, setV, sc32, -2, 2);

    StringSet<String<AminoAcid>> pH, pV;
    appendValue(pH, "MKVLAAGIVGLLLA");
    appendValue(pV, "MKVIAAGLVGLA");
    Score<int16_t, ScoreMatrix<AminoAcid, ScoreSpecBlosum62>> blosum(-1, -11);
    String<int16_t> h = localAlignmentScore(gpu, pH, pV, blosum);

    typedef Gaps<Dna5String> TGaps;
    StringSet<TGaps> gapsH, gapsV;
    for (size_t k = 0; k < length(setH); ++k) {
        appendValue(gapsH, TGaps(setH[k]));
        appendValue(gapsV, TGaps(setV[k]));
    }
    String<int16_t> i = globalAlignment(gpu, gapsH, gapsV, sc16);
    String<int16_t> j = globalAlignment(gpu, gapsH, gapsV, sc16, AlignConfig<false, true, true, false>());
    String<int> k = globalAlignment(gpu, gapsH, gapsV, sc32, -4, 4);
    String<int> l = localAlignment(gpu, gapsH, gapsV, sc32);
    String<int> m = localAlignment(gpu, gapsH, gapsV, sc32, -4, 4);

    typedef Align<Dna5String> TAlign;
    StringSet<TAlign> aligns;
    for (size_t q = 0; q < length(setH); ++q) {
        TAlign al;
        resize(rows(al), 2);
        assignSource(row(al, 0), setH[q]);
        assignSource(row(al, 1), setV[q]);
        appendValue(aligns, al);
    }
    String<int16_t> n1 = globalAlignment(gpu, aligns, sc16);
    String<int> n2 = globalAlignment(gpu, aligns, sc32, AlignConfig<true, false, false, true>(), -3, 5);
    String<int> n3 = localAlignment(gpu, aligns, sc32);
    String<int> n4 = localAlignment(gpu, aligns, sc32, -2, 2);

    std::cout << a[0] << ' ' << b[0] << ' ' << c[0] << ' ' << d[0] << ' ' << e[1] << ' ' << f[0] << ' ' << g[0] << ' '
              << h[0] << ' ' << i[0] << ' ' << j[0] << ' ' << k[0] << ' ' << l[0] << ' ' << m[0] << ' ' << n1[0] << ' '
              << n2[0] << ' ' << n3[0] << ' ' << n4[0] << '\n'
              << gapsH[0] << '\n' << gapsV[0] << '\n' << aligns[0] << '\n';
    seeds_demo(gpu);
    io_demo(gpu);
    return 0;
}
