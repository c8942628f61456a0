"""The GPU aligner in the shape of the editor's alignment-tool plugin.

tweakseq/Core/AlignmentTool.h:36-71 defines what the editor asks of a tool:
name, version, executable path, a preferred flag, whether the result comes
on stdout, `makeCommand(fin, fout, exec, args)` and XML settings
(`<alignment_tool><name/><path/><preferred/></alignment_tool>`, as
tweakseq/Core/Muscle.cpp:54-86 writes them).  GpuAlignmentTool answers the
same calls; its executable is the `tsq_align` program built with the
library, which takes the editor's FASTA and writes the gapped FASTA that
Project::readNewAlignment reads back.  `align_files` runs that command
in-process instead of through QProcess.
"""
from __future__ import annotations

import subprocess
import xml.etree.ElementTree as ET

from . import build as _build


class GpuAlignmentTool:
    def __init__(self):
        self._name = "tweakseq-gb300"
        self._version = "1"
        self._executable = _build.CLI
        self._preferred = False
        self._uses_stdout = False

    # Accessors of AlignmentTool.h:43-55.
    def name(self) -> str:
        return self._name

    def version(self) -> str:
        return self._version

    def executable(self) -> str:
        return self._executable

    def setExecutable(self, e: str) -> None:
        self._executable = e

    def setPreferred(self, pref: bool) -> None:
        self._preferred = bool(pref)

    def preferred(self) -> bool:
        return self._preferred

    def usesStdOut(self) -> bool:
        return self._uses_stdout

    def makeCommand(self, fin: str, fout: str, local: bool = False, dna: bool = False) -> tuple[str, list[str]]:
        """(exec, args) for aligning the FASTA in fin into fout, as the
        editor's tools build them (MUSCLE-style -in/-out)."""
        args = ["-in", fin, "-out", fout]
        if local:
            args.append("--local")
        if dna:
            args.append("--dna")
        return self._executable, args

    def writeSettings(self, parent: ET.Element) -> ET.Element:
        elem = ET.SubElement(parent, "alignment_tool")
        ET.SubElement(elem, "name").text = self._name
        ET.SubElement(elem, "path").text = self._executable
        ET.SubElement(elem, "preferred").text = "yes" if self._preferred else "no"
        return elem

    def readSettings(self, doc: ET.Element) -> None:
        for node in doc.iter("alignment_tool"):
            fields = {child.tag: (child.text or "") for child in node}
            if fields.get("name") != self._name:
                continue
            if "path" in fields:
                self._executable = fields["path"]
            if "preferred" in fields:
                self._preferred = fields["preferred"] == "yes"

    def align_files(self, fin: str, fout: str, **kw) -> subprocess.CompletedProcess:
        exe, args = self.makeCommand(fin, fout, **kw)
        return subprocess.run([exe, *args], capture_output=True, text=True)
