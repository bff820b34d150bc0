"""The reference's command flags and REMDConfig.txt, read by the host library
(no GPU).  Semantics follow InputData's flag loop (src/Initialization.c:63-256)
and the sREMD launcher (src/REMDExec.c:79-118)."""
import pytest

from sdmd_gb300.host import OUT_NAMES, parse_args, read_remd_config


def test_flags_as_the_reference_reads_them(tmp_path):
    (tmp_path / "in").mkdir()
    (tmp_path / "out").mkdir()
    c = parse_args(["sDMD", "-f", "ala10.gro", "-i", str(tmp_path / "in"), "-o", str(tmp_path / "out"),
                    "-pot", "-kin", "energy_kin.txt", "-tem", "-pdb", "traj.pdb", "-box", "40", "41.5", "42",
                    "-si", "restart.dat", "-so", "next.dat", "-pre", "-his", "-COM", "stray"])
    assert c.coordinate_file == b"ala10.gro"
    assert c.datadir.decode() == str(tmp_path / "in") and c.savedir.decode() == str(tmp_path / "out")
    on = {OUT_NAMES[k]: c.out_on[k] for k in range(len(OUT_NAMES))}
    names = {OUT_NAMES[k]: c.out_name[k].value for k in range(len(OUT_NAMES))}
    assert on["pot"] and on["kin"] and on["tem"] and not on["HBn"]
    assert names["kin"] == b"energy_kin.txt" and names["pot"] == b"" and names["saved"] == b"next.dat"
    # -pdb names the pdb file but switches the xyz output on, as the reference does
    assert names["pdb"] == b"traj.pdb" and on["xyz"] and not on["pdb"]
    assert c.box_given and list(c.box) == [40.0, 41.5, 42.0]
    assert c.saved_in == b"restart.dat" and c.pre_bonds == 1
    assert list(c.charge) == [0, 0, 0, 1, 0, 0, 0, 0, 1]


def test_defaults_and_optional_names():
    c = parse_args(["sDMD", "-f", "-pot"])           # -f followed by a flag keeps the default name
    assert c.coordinate_file == b"coordinate.gro" and c.saved_in == b"savedData.dat"
    assert c.out_on[OUT_NAMES.index("pot")] == 1


def test_remd_flag_and_its_saved_data_name():
    c = parse_args(["sDMD", "-REMD", "localhost", "20202", "0.469974", "3", "50", "_r3"])
    assert c.remd == 1 and c.remd_server == b"localhost" and c.remd_port == 20202
    assert c.remd_T == 0.469974 and c.remd_num == 3 and c.remd_rate == 50
    assert c.saved_in == b"savedData_r3.dat"
    with pytest.raises(ValueError, match="temperature value"):
        parse_args(["sDMD", "-REMD", "localhost", "20202"])


def test_invalid_directories_are_refused(tmp_path):
    with pytest.raises(ValueError, match="-i"):
        parse_args(["sDMD", "-i", str(tmp_path / "missing")])
    with pytest.raises(ValueError, match="-o"):
        parse_args(["sDMD", "-o"])


def test_help_flag():
    assert parse_args(["sDMD", "-h"]).help == 1


CONFIG = """#REPLICA EXCHANGE MD CONFIGURATION FILE
ReplicaNum              = 4
Temperatures            = 236.5 250 263.5 416
SocketPort              = 20202
ExchangeRate            = 50.7
"""


def test_remd_config_gives_each_replica_the_launchers_temperature(tmp_path):
    p = tmp_path / "REMDConfig.txt"
    p.write_text(CONFIG)
    cfg = read_remd_config(p)
    assert cfg["n"] == 4 and cfg["port"] == 20202
    assert cfg["exchange_time"] == 50.0              # the replica reads the rate with atoi
    assert cfg["T_kelvin"] == [236.5, 250.0, 263.5, 416.0]
    # the launcher prints T * BOLTZMANN with "%lf"; the replica reads that text back
    assert list(cfg["T"]) == [float("%lf" % (t * 0.0019872041)) for t in (236.5, 250.0, 263.5, 416.0)]
    assert list(cfg["num"]) == [1, 2, 3, 4]


@pytest.mark.parametrize("temps,msg", [("236.5 250 263.5", "less"), ("236.5 250 263.5 300 416", "larger")])
def test_remd_config_count_mismatch_is_refused(tmp_path, temps, msg):
    p = tmp_path / "REMDConfig.txt"
    p.write_text(CONFIG.replace("236.5 250 263.5 416", temps))
    with pytest.raises(ValueError, match=msg):
        read_remd_config(p)
