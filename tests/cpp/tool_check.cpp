// tool_check -- exercises tweakseq_gb300_tool.hpp, the in-process form of
// the alignment tool.
//
//   tool_check --host              the parts that need no GPU: the FASTA
//                                  reader (labels, comments, gaps, case),
//                                  the 80-column writer, the settings XML
//                                  round trip, makeCommand; prints "host ok"
//   tool_check FIN FOUT [--local] [--dna]
//                                  alignFile(FIN, FOUT) with those options;
//                                  prints the status name
#include <cstdio>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "tweakseq_gb300_tool.hpp"

namespace {

int failures = 0;

void expect(bool ok, const char *what) {
  if (!ok) {
    std::fprintf(stderr, "FAILED: %s\n", what);
    ++failures;
  }
}

int host_checks() {
  using tsq_tool::GpuAlignmentTool;
  using tsq_tool::Record;
  // FASTA as the editor writes and reads it.
  std::istringstream in(
      "  \n>seqA some description\n;a comment\n;another\nacde--fg\n  HIK. \n;not a comment here\n>seqB\nmnp\n");
  std::vector<Record> recs;
  std::string err;
  expect(tsq_tool::read_fasta(in, recs, err), "read_fasta succeeds");
  expect(recs.size() == 3, "three records (';' after sequence lines starts one)");
  if (recs.size() == 3) {
    expect(recs[0].header == ">seqA some description", "header kept whole");
    expect(recs[0].label == "seqA", "label up to the first space");
    expect(recs[0].residues == "ACDEFGHIK", "gaps dropped, upper case");
    expect(recs[2].residues == "MNP", "last record");
  }
  std::istringstream empty("no records here\n");
  std::vector<Record> none;
  expect(!tsq_tool::read_fasta(empty, none, err), "no records is an error");
  // 80 residues per line.
  std::ostringstream out;
  tsq_tool::write_wrapped(out, ">x", std::string(170, 'A'));
  expect(out.str() == ">x\n" + std::string(80, 'A') + "\n" + std::string(80, 'A') + "\n" + std::string(10, 'A') + "\n",
         "80-column wrapping");
  // Settings and command.
  GpuAlignmentTool t("/opt/tsq_align");
  expect(t.name() == "tweakseq-gb300" && !t.usesStdOut() && !t.preferred(), "identity of the tool");
  t.setPreferred(true);
  const std::string xml = "<settings>" +
                          std::string("<alignment_tool><name>muscle</name><path>/usr/bin/muscle</path>"
                                      "<preferred>no</preferred></alignment_tool>") +
                          t.settingsXml() + "</settings>";
  GpuAlignmentTool u("tsq_align");
  expect(u.readSettingsXml(xml), "own settings found among other tools'");
  expect(u.executable() == "/opt/tsq_align" && u.preferred(), "path and preferred flag read back");
  std::string exec;
  std::vector<std::string> args;
  u.options.local = true;
  u.makeCommand("in.fa", "out.fa", exec, args);
  expect(exec == "/opt/tsq_align", "command executable");
  expect(args == std::vector<std::string>({"-in", "in.fa", "-out", "out.fa", "--local"}), "command arguments");
  if (failures == 0) std::printf("host ok\n");
  return failures == 0 ? 0 : 1;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc > 1 && std::strcmp(argv[1], "--host") == 0) return host_checks();
  if (argc < 3) {
    std::fprintf(stderr, "usage: tool_check --host | FIN FOUT [--local] [--dna]\n");
    return 2;
  }
  tsq_tool::GpuAlignmentTool tool;
  for (int k = 3; k < argc; ++k) {
    if (std::strcmp(argv[k], "--local") == 0) tool.options.local = true;
    if (std::strcmp(argv[k], "--dna") == 0) {
      tool.options.dna = true;
      tool.options.gap_open = 5;
      tool.options.gap_extend = 2;
    }
  }
  std::string err;
  const int rc = tool.alignFile(argv[1], argv[2], err);
  std::printf("%s\n", tsq_tool::status_name(rc));
  if (rc != TSQ_OK) std::fprintf(stderr, "%s\n", err.c_str());
  return rc == TSQ_OK ? 0 : 1;
}
