"""Test-only stand-in for the reference core's flat-table I/O (ROOT files through uproot, absent here): the names the
CRV modules import, with readers that refuse."""
DIR = "dump"
KEY = ["run", "subrun", "event"]
PRIMARY_MUON_PDG = 13


def _absent(*a, **k):
    raise RuntimeError("ROOT table I/O (uproot) is not available in this environment")


expand = livetime = primary_muons = read = read_many = write = _absent
