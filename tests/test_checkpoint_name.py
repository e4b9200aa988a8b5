"""The reference's checkpoint file naming (basic_IMSRG.f90:3142-3160), a
host-only entry point of the library (no GPU needed)."""
import pytest


@pytest.mark.parametrize("prefix,s,expect", [
    ("O16_hw20_e6", 2.5, "scratch/O16_hw20_s2.5000.bin"),
    ("O16_hw20_e6", 12.5, "scratch/O16_hw20_s12.500.bin"),
    ("He4_hw16eMax2", 0.5, "scratch/He4_hw16_s0.5000.bin"),
    ("nohwfield", 50.0, "scratch/nohwfi_s50.000.bin"),
    ("plainprefix", 7.0, "scratch/plainprefix_s7.0000.bin"),
])
def test_checkpoint_name(gpu_lib_cpu, prefix, s, expect):
    assert gpu_lib_cpu.checkpoint_name("scratch/", prefix, s) == expect
