// tsq_align -- command-line front end of the GB300 alignment library, a
// drop-in for the external aligner behind the editor's AlignmentTool seam.
//
// The editor writes the sequences to align as FASTA and runs
// `<exec> <args>` built by AlignmentTool::makeCommand, reading the gapped
// result back as FASTA (tweakseq/Core/AlignmentTool.h:36-71,
// tweakseq/UI/SeqEditMainWin.cpp:1616-1663, Project::readNewAlignment in
// tweakseq/Core/Project.cpp:908-1032).  This program accepts the same shapes
// of command line as the tools the editor knows (MUSCLE-style `-in F -out
// F`, ClustalO-style `-i F -o F`, or output on stdout as MAFFT does) and:
//
//   two sequences  -> their pairwise alignment as gapped FASTA, same labels
//                     and header lines, 80 residues per line (the editor's
//                     own FASTA writer wraps at 80, FASTAFile.cpp:149-171);
//                     with --local each row still holds its whole input
//                     sequence: the unaligned flanks stand against gaps
//                     around the aligned core (full_local_rows in
//                     tweakseq_gb300_tool.hpp, which also holds the FASTA
//                     reader and writer shared with the in-process tool);
//   --all-vs-all   -> every unordered pair, one TSV line per pair: labels,
//                     score, identical columns, columns, percent identity
//                     (the distance input of a guide tree);
//   --tree upgma|nj -> the guide tree of the sequences from their all-vs-all
//                     identities, as Newick text (branch lengths in
//                     distance units, distance = 1 - identity);
//   --consensus    -> the input is an alignment (equal-length gapped rows,
//                     kept as they are); one FASTA record with the consensus
//                     line the editor draws (Consensus::calculate,
//                     tweakseq/Core/Annotations/Consensus.cpp:80-161).
//
// FASTA is read as the editor reads it (FASTAFile.cpp:71-147): a record
// starts at '>' or ';', its label is the header text up to the first space,
// further ';' lines right after a header are comments, sequence lines are
// concatenated.  Gap characters already in the input ('-', '.') are dropped
// and residues upper-cased, as the external aligners do with editor output
// (except for --consensus, which reads the rows verbatim).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/tweakseq_gb300.h"
#include "../../include/tweakseq_gb300_tool.hpp"

namespace {

using tsq_tool::full_local_rows;
using tsq_tool::read_fasta;
using tsq_tool::Record;
using tsq_tool::status_name;
using tsq_tool::write_wrapped;

void usage() {
  std::fprintf(stderr,
               "usage: tsq_align [-in|-i FILE] [-out|-o FILE] [--local] [--dna | --matrix blosum62|dna]\n"
               "                 [--gap-open N] [--gap-extend N] [--all-vs-all | --tree upgma|nj | --consensus]\n"
               "  Two sequences: gapped FASTA of their alignment (stdout when no output file).\n"
               "  --all-vs-all: TSV of every pair (label_a, label_b, score, n_ident, n_cols, identity %%).\n"
               "  --tree: Newick guide tree from all-vs-all identities (UPGMA or neighbour joining).\n"
               "  --consensus: consensus line of an alignment (equal-length rows) as one FASTA record.\n");
}

// Newick text of the joins (leaves 0..n-1, join t is node n + t).
std::string newick(const std::vector<tsq_tree_node> &nodes, const std::vector<Record> &recs) {
  const int n = int(recs.size());
  std::vector<std::string> text(size_t(2 * n - 1));
  for (int k = 0; k < n; ++k) text[size_t(k)] = recs[size_t(k)].label;
  for (int t = 0; t < n - 1; ++t) {
    const tsq_tree_node &nd = nodes[size_t(t)];
    char la[64], lb[64];
    std::snprintf(la, sizeof(la), ":%.6f", double(nd.left_length) / 4294967296.0);
    std::snprintf(lb, sizeof(lb), ":%.6f", double(nd.right_length) / 4294967296.0);
    text[size_t(n + t)] = "(" + text[size_t(nd.left)] + la + "," + text[size_t(nd.right)] + lb + ")";
  }
  return (n == 1 ? text[0] : text[size_t(2 * n - 2)]) + ";";
}

}  // namespace

int main(int argc, char **argv) {
  std::string fin, fout;
  tsq_params p{};
  p.matrix = TSQ_MATRIX_BLOSUM62;
  p.gap_open = 11;
  p.gap_extend = 1;
  p.mode = TSQ_GLOBAL;
  p.output = TSQ_OUT_ALIGNMENT;
  p.lane = TSQ_LANE_AUTO;
  bool all_vs_all = false, gaps_set = false, consensus = false;
  int tree = -1;
  for (int k = 1; k < argc; ++k) {
    const std::string a = argv[k];
    auto next = [&](const char *what) -> std::string {
      if (k + 1 >= argc) {
        std::fprintf(stderr, "tsq_align: %s needs a value\n", what);
        std::exit(2);
      }
      return argv[++k];
    };
    if (a == "-in" || a == "-i" || a == "--in") fin = next("-in");
    else if (a == "-out" || a == "-o" || a == "--out") fout = next("-out");
    else if (a == "--local") p.mode = TSQ_LOCAL;
    else if (a == "--dna") p.matrix = TSQ_MATRIX_DNA;
    else if (a == "--matrix") {
      const std::string m = next("--matrix");
      if (m == "blosum62") p.matrix = TSQ_MATRIX_BLOSUM62;
      else if (m == "dna") p.matrix = TSQ_MATRIX_DNA;
      else {
        std::fprintf(stderr, "tsq_align: unknown matrix %s\n", m.c_str());
        return 2;
      }
    } else if (a == "--gap-open") {
      p.gap_open = std::atoi(next("--gap-open").c_str());
      gaps_set = true;
    } else if (a == "--gap-extend") {
      p.gap_extend = std::atoi(next("--gap-extend").c_str());
      gaps_set = true;
    } else if (a == "--all-vs-all") all_vs_all = true;
    else if (a == "--consensus") consensus = true;
    else if (a == "--tree") {
      const std::string m = next("--tree");
      if (m == "upgma") tree = TSQ_TREE_UPGMA;
      else if (m == "nj") tree = TSQ_TREE_NJ;
      else {
        std::fprintf(stderr, "tsq_align: unknown tree method %s\n", m.c_str());
        return 2;
      }
    }
    else if (a == "-h" || a == "--help") {
      usage();
      return 0;
    } else if (fin.empty() && a[0] != '-') fin = a;  // MAFFT style: input file as the last argument
    else {
      std::fprintf(stderr, "tsq_align: unknown argument %s\n", a.c_str());
      usage();
      return 2;
    }
  }
  if (p.matrix == TSQ_MATRIX_DNA && !gaps_set) {
    p.gap_open = 5;
    p.gap_extend = 2;
  }
  std::vector<Record> recs;
  std::string err;
  {
    std::ifstream f;
    std::istream *in = &std::cin;
    if (!fin.empty()) {
      f.open(fin);
      if (!f) {
        std::fprintf(stderr, "tsq_align: cannot open %s\n", fin.c_str());
        return 1;
      }
      in = &f;
    }
    if (!read_fasta(*in, recs, err, consensus)) {
      std::fprintf(stderr, "tsq_align: %s\n", err.c_str());
      return 1;
    }
  }
  std::ofstream fo;
  std::ostream *out = &std::cout;
  if (!fout.empty()) {
    fo.open(fout);
    if (!fo) {
      std::fprintf(stderr, "tsq_align: cannot write %s\n", fout.c_str());
      return 1;
    }
    out = &fo;
  }

  if (consensus) {
    const size_t cols = recs[0].residues.size();
    std::string rows;
    for (const Record &r : recs) {
      if (r.residues.size() != cols) {
        std::fprintf(stderr, "tsq_align: --consensus needs rows of equal length (%s has %zu, not %zu)\n",
                     r.label.c_str(), r.residues.size(), cols);
        return 1;
      }
      rows += r.residues;
    }
    std::string cons(cols, '?');
    const int rc = tsq_consensus(reinterpret_cast<const uint8_t *>(rows.data()), int32_t(recs.size()),
                                 int32_t(cols), int64_t(cols), -1.0, reinterpret_cast<uint8_t *>(&cons[0]), nullptr,
                                 nullptr);
    if (rc != TSQ_OK) {
      std::fprintf(stderr, "tsq_align: %s\n", status_name(rc));
      return 1;
    }
    write_wrapped(*out, ">consensus", cons);
    return 0;
  }

  if (!all_vs_all && tree < 0) {
    if (recs.size() != 2) {
      std::fprintf(stderr, "tsq_align: pairwise alignment needs exactly 2 sequences (got %zu); "
                           "use --all-vs-all for more\n",
                   recs.size());
      return 1;
    }
    tsq_result r;
    const std::string &a = recs[0].residues, &b = recs[1].residues;
    const int rc = tsq_align_pair(reinterpret_cast<const uint8_t *>(a.data()), int32_t(a.size()),
                                  reinterpret_cast<const uint8_t *>(b.data()), int32_t(b.size()), &p, &r);
    if (rc != TSQ_OK) {
      std::fprintf(stderr, "tsq_align: %s\n", status_name(rc));
      return 1;
    }
    if (p.mode == TSQ_LOCAL) {
      // The editor replaces each sequence's residues with the row it reads
      // back (Project::readNewAlignment, tweakseq/Core/Project.cpp:1016), so
      // a row must hold the whole input sequence.  Full-length local rows:
      // a's unaligned prefix against gaps, then b's unaligned prefix against
      // gaps, the aligned core, a's unaligned suffix against gaps, then b's
      // unaligned suffix against gaps.
      std::string row_a, row_b;
      full_local_rows(a, b, r, row_a, row_b);
      write_wrapped(*out, recs[0].header, row_a);
      write_wrapped(*out, recs[1].header, row_b);
    } else {
      write_wrapped(*out, recs[0].header, r.aln_a);
      write_wrapped(*out, recs[1].header, r.aln_b);
    }
    tsq_result_free(&r);
    return 0;
  }

  // All-vs-all: one residue buffer, every unordered pair, identity output.
  std::string buf;
  std::vector<int64_t> off;
  for (const Record &r : recs) {
    off.push_back(int64_t(buf.size()));
    buf += r.residues;
  }
  std::vector<tsq_pair_desc> pairs;
  for (size_t x = 0; x < recs.size(); ++x)
    for (size_t y = x + 1; y < recs.size(); ++y)
      pairs.push_back(tsq_pair_desc{off[x], off[y], int32_t(recs[x].residues.size()),
                                    int32_t(recs[y].residues.size())});
  p.output = TSQ_OUT_IDENTITY;
  std::vector<tsq_result> res(pairs.size());
  tsq_batch_opts o{-1, 0, 0, 0};
  const int rc = tsq_align_batch(reinterpret_cast<const uint8_t *>(buf.data()), int64_t(buf.size()), pairs.data(),
                                 int64_t(pairs.size()), &p, &o, res.data());
  if (rc != TSQ_OK) {
    std::fprintf(stderr, "tsq_align: %s\n", status_name(rc));
    return 1;
  }
  if (tree >= 0) {
    std::vector<int32_t> ident(res.size()), ncols(res.size());
    for (size_t k = 0; k < res.size(); ++k) {
      ident[k] = res[k].n_ident;
      ncols[k] = res[k].n_cols;
    }
    std::vector<tsq_tree_node> nodes(recs.size() > 1 ? recs.size() - 1 : 1);
    const int trc = tsq_guide_tree(int32_t(recs.size()), ident.data(), ncols.data(), tree, nodes.data());
    if (trc != TSQ_OK) {
      std::fprintf(stderr, "tsq_align: %s\n", status_name(trc));
      return 1;
    }
    nodes.resize(recs.size() - 1);
    *out << newick(nodes, recs) << '\n';
    return 0;
  }
  *out << "label_a\tlabel_b\tscore\tn_ident\tn_cols\tidentity_pct\n";
  size_t k = 0;
  for (size_t x = 0; x < recs.size(); ++x)
    for (size_t y = x + 1; y < recs.size(); ++y, ++k) {
      const tsq_result &r = res[k];
      char pct[32];
      std::snprintf(pct, sizeof(pct), "%.2f", r.n_cols > 0 ? 100.0 * r.n_ident / r.n_cols : 0.0);
      *out << recs[x].label << '\t' << recs[y].label << '\t' << r.score << '\t' << r.n_ident << '\t' << r.n_cols
           << '\t' << pct << '\n';
    }
  return 0;
}
