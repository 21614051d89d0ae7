"""iterateMC's summary.out (source/iteration_mod.f90:1316-1350) from iteration reports: four records per
iteration with the truncated percentages, rewritten at the first iteration and appended to after."""
from mocassin_xray_gb300.iterate import IterationReport
from mocassin_xray_gb300.output import write_summary


def _report(it, conv, hit, ion, te):
    return IterationReport(iteration=it, n_photons=1000, conv_percent=conv, no_hit_percent=hit,
                           no_ion_bal_percent=ion, no_te_bal_percent=te, te_change_max=0.0, te_change_mean=0.0,
                           ms={}, wall_s=0.0, transport={})


def test_summary_records(tmp_path):
    p = tmp_path / "summary.out"
    write_summary(p, _report(1, 12.9, 3.99, 0.5, 40.0))
    write_summary(p, _report(2, 95.2, 0.0, 0.0, 1.7))
    lines = p.read_text().splitlines()
    assert len(lines) == 8
    assert all(l.startswith(" ! iterateMC: [Summary] Iteration ") for l in lines)
    fields = [l.split() for l in lines]
    # iteration, the truncated percentage, the grid
    assert [(int(f[4]), int(f[6]), int(f[-1])) for f in fields] == [
        (1, 12, 1), (1, 3, 1), (1, 0, 1), (1, 40, 1), (2, 95, 1), (2, 0, 1), (2, 0, 1), (2, 1, 1)]
    assert "conveged cells in grid" in lines[0] and "Te balance not reached in grid" in lines[3]
    # a new run starts the file again
    write_summary(p, _report(1, 50.0, 0.0, 0.0, 0.0))
    assert len(p.read_text().splitlines()) == 4
