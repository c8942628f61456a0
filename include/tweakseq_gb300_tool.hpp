/* tweakseq_gb300_tool.hpp -- the GPU aligner as an in-process alignment
 * tool, in plain C++17 (no Qt).
 *
 * The editor drives an aligner through AlignmentTool
 * (tweakseq/Core/AlignmentTool.h:36-71): name, version, executable path,
 * preferred flag, whether the result comes on stdout, makeCommand(fin, fout,
 * exec, args) and XML settings; it writes the selected sequences as FASTA,
 * runs the command (tweakseq/UI/SeqEditMainWin.cpp:1616-1663) and reads the
 * gapped FASTA back (Project::readNewAlignment,
 * tweakseq/Core/Project.cpp:908-1032).  GpuAlignmentTool answers the same
 * calls -- its executable is the tsq_align program built with the library --
 * and alignFile() does in process what that program does for two
 * sequences: it reads the FASTA with the editor's rules
 * (tweakseq/Core/FASTAFile.cpp:71-147), aligns through tsq_align_pair and
 * writes the gapped rows, 80 residues per line (FASTAFile.cpp:149-171).  A
 * Qt subclass of AlignmentTool needs only to convert QString to and from
 * std::string around these calls.
 *
 * Local mode keeps every residue: each output row is its whole input
 * sequence, the unaligned flanks standing against gaps around the aligned
 * core (full_local_rows), because readNewAlignment replaces each sequence's
 * residues with its row. */
#pragma once

#include <cctype>
#include <cstdio>
#include <fstream>
#include <istream>
#include <ostream>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "tweakseq_gb300.h"

namespace tsq_tool {

struct Record {
  std::string header;  // the whole header line, '>' included
  std::string label;   // the header text up to the first space
  std::string residues;
};

/* Reads FASTA as the editor does: a record starts at '>' or ';', its label
 * is the header up to the first space, further ';' lines right after a
 * header are comments, sequence lines are concatenated with white space
 * removed.  Unless verbatim, gap characters ('-', '.') are dropped and
 * residues upper-cased, as the external aligners treat editor output. */
inline bool read_fasta(std::istream &in, std::vector<Record> &out, std::string &err, bool verbatim = false) {
  std::string line;
  enum { kSeek, kComment, kSequence } state = kSeek;
  while (std::getline(in, line)) {
    size_t a = 0, b = line.size();
    while (a < b && std::isspace(static_cast<unsigned char>(line[a]))) ++a;
    while (b > a && std::isspace(static_cast<unsigned char>(line[b - 1]))) --b;
    line = line.substr(a, b - a);
    if (line.empty()) continue;
    const char c = line[0];
    if (c == '>' || c == ';') {
      if (state == kComment && c == ';') continue;  // further comment lines
      Record r;
      r.header = line;
      const size_t sp = line.find(' ', 1);
      r.label = sp == std::string::npos ? line.substr(1) : line.substr(1, sp - 1);
      out.push_back(r);
      state = kComment;
      continue;
    }
    if (state == kSeek) continue;
    for (char ch : line) {
      if (std::isspace(static_cast<unsigned char>(ch))) continue;
      if (verbatim) {
        out.back().residues.push_back(ch);
        continue;
      }
      if (ch == '-' || ch == '.') continue;
      out.back().residues.push_back(char(std::toupper(static_cast<unsigned char>(ch))));
    }
    state = kSequence;
  }
  if (out.empty()) {
    err = "no FASTA records";
    return false;
  }
  return true;
}

/* One FASTA record, 80 residues per line. */
inline void write_wrapped(std::ostream &o, const std::string &header, const std::string &s) {
  o << header << '\n';
  for (size_t k = 0; k < s.size(); k += 80) o << s.substr(k, 80) << '\n';
}

/* Full-length rows of a local alignment: every residue of a and of b
 * appears in its row, in order, so that removing the gaps gives the input
 * back.  Columns, left to right: a[0:a_begin] over gaps, gaps over
 * b[0:b_begin], the aligned core (aln_a over aln_b), a[a_end:] over gaps,
 * gaps over b[b_end:].  An empty local alignment (score 0, coordinates 0)
 * gives a over gaps followed by gaps over b. */
inline void full_local_rows(const std::string &a, const std::string &b, const tsq_result &r, std::string &row_a,
                            std::string &row_b) {
  const size_t ab = size_t(r.a_begin), ae = size_t(r.a_end), bb = size_t(r.b_begin), be = size_t(r.b_end);
  const std::string core_a = r.aln_a ? r.aln_a : "", core_b = r.aln_b ? r.aln_b : "";
  row_a = a.substr(0, ab) + std::string(bb, '-') + core_a + a.substr(ae) + std::string(b.size() - be, '-');
  row_b = std::string(ab, '-') + b.substr(0, bb) + core_b + std::string(a.size() - ae, '-') + b.substr(be);
}

inline const char *status_name(int rc) {
  switch (rc) {
    case TSQ_OK: return "ok";
    case TSQ_E_INVALID_ARG: return "invalid argument";
    case TSQ_E_INVALID_RESIDUE: return "invalid residue for the scoring matrix";
    case TSQ_E_NOMEM: return "out of memory";
    case TSQ_E_CUDA: return "CUDA error (no usable GPU?)";
    case TSQ_E_TOO_LARGE: return "input too large";
    default: return "error";
  }
}

/* Scoring of the tool (the editor's tools carry theirs in their settings). */
struct Options {
  bool local = false;
  bool dna = false;  // DNA +2/-3 instead of BLOSUM62
  int gap_open = 11, gap_extend = 1;
};

class GpuAlignmentTool {
 public:
  explicit GpuAlignmentTool(std::string executable = "tsq_align") : executable_(std::move(executable)) {}

  /* The accessors of AlignmentTool.h:43-55. */
  const std::string &name() const { return name_; }
  const std::string &version() const { return version_; }
  const std::string &executable() const { return executable_; }
  void setExecutable(const std::string &e) { executable_ = e; }
  void setPreferred(bool pref) { preferred_ = pref; }
  bool preferred() const { return preferred_; }
  bool usesStdOut() const { return false; }

  /* The command an editor runs for the out-of-process form: tsq_align with
   * MUSCLE-style -in/-out (AlignmentTool::makeCommand). */
  void makeCommand(const std::string &fin, const std::string &fout, std::string &exec,
                   std::vector<std::string> &args) const {
    exec = executable_;
    args = {"-in", fin, "-out", fout};
    if (options.local) args.push_back("--local");
    if (options.dna) args.push_back("--dna");
  }

  /* XML settings in the shape the editor's tools write
   * (<alignment_tool><name/><path/><preferred/></alignment_tool>,
   * tweakseq/Core/Muscle.cpp:54-86). */
  std::string settingsXml() const {
    return "<alignment_tool><name>" + name_ + "</name><path>" + executable_ + "</path><preferred>" +
           (preferred_ ? "yes" : "no") + "</preferred></alignment_tool>";
  }
  /* Reads the path and preferred flag of the first <alignment_tool> element
   * named as this tool; false when there is none. */
  bool readSettingsXml(const std::string &xml) {
    size_t at = 0;
    for (;;) {
      const size_t b = xml.find("<alignment_tool>", at);
      if (b == std::string::npos) return false;
      const size_t e = xml.find("</alignment_tool>", b);
      if (e == std::string::npos) return false;
      const std::string body = xml.substr(b, e - b);
      if (field(body, "name") == name_) {
        const std::string path = field(body, "path"), pref = field(body, "preferred");
        if (!path.empty()) executable_ = path;
        if (!pref.empty()) preferred_ = pref == "yes";
        return true;
      }
      at = e;
    }
  }

  /* Aligns two residue strings (already filtered: letters only) and returns
   * the two gapped rows, whole sequences in local mode. */
  int alignPair(const std::string &a, const std::string &b, std::string &row_a, std::string &row_b,
                int32_t *score = nullptr) const {
    tsq_params p{};
    p.matrix = options.dna ? TSQ_MATRIX_DNA : TSQ_MATRIX_BLOSUM62;
    p.gap_open = options.gap_open;
    p.gap_extend = options.gap_extend;
    p.mode = options.local ? TSQ_LOCAL : TSQ_GLOBAL;
    p.output = TSQ_OUT_ALIGNMENT;
    p.lane = TSQ_LANE_AUTO;
    tsq_result r{};
    const int rc = tsq_align_pair(reinterpret_cast<const uint8_t *>(a.data()), int32_t(a.size()),
                                  reinterpret_cast<const uint8_t *>(b.data()), int32_t(b.size()), &p, &r);
    if (rc != TSQ_OK) return rc;
    if (options.local) {
      full_local_rows(a, b, r, row_a, row_b);
    } else {
      row_a = r.aln_a ? r.aln_a : "";
      row_b = r.aln_b ? r.aln_b : "";
    }
    if (score) *score = r.score;
    tsq_result_free(&r);
    return TSQ_OK;
  }

  /* What the external program does for "Align selection": the two FASTA
   * records of fin, aligned, written to fout as gapped FASTA with their
   * header lines.  Returns TSQ_OK or an error code (message in err). */
  int alignFile(const std::string &fin, const std::string &fout, std::string &err) const {
    std::ifstream in(fin);
    if (!in) {
      err = "cannot read " + fin;
      return TSQ_E_INVALID_ARG;
    }
    std::vector<Record> recs;
    if (!read_fasta(in, recs, err)) return TSQ_E_INVALID_ARG;
    if (recs.size() != 2) {
      err = "two sequences expected, got " + std::to_string(recs.size());
      return TSQ_E_INVALID_ARG;
    }
    std::string row_a, row_b;
    const int rc = alignPair(recs[0].residues, recs[1].residues, row_a, row_b);
    if (rc != TSQ_OK) {
      err = status_name(rc);
      return rc;
    }
    std::ofstream out(fout);
    if (!out) {
      err = "cannot write " + fout;
      return TSQ_E_INVALID_ARG;
    }
    write_wrapped(out, recs[0].header, row_a);
    write_wrapped(out, recs[1].header, row_b);
    return out ? TSQ_OK : TSQ_E_INVALID_ARG;
  }

  Options options;

 private:
  static std::string field(const std::string &body, const std::string &tag) {
    const std::string open = "<" + tag + ">", close = "</" + tag + ">";
    const size_t b = body.find(open);
    if (b == std::string::npos) return "";
    const size_t e = body.find(close, b);
    if (e == std::string::npos) return "";
    return body.substr(b + open.size(), e - b - open.size());
  }

  std::string name_ = "tweakseq-gb300";
  std::string version_ = "1";
  std::string executable_;
  bool preferred_ = false;
};

}  // namespace tsq_tool
