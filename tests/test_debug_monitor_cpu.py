"""DebugMonitor configuration and result reader (CPU)."""
import pytest

from neuronbridge_gb300 import DebugMonitorConfig, DebugMonitorResult, open_debug_monitor


def test_config_defaults_match_reference_fields():
    c = DebugMonitorConfig()
    d = c.to_dict()
    assert d["output_dir"] == "debug_monitor" and d["sample_interval_steps"] == 1 and d["flush_interval_steps"] == 100
    assert d["record_spikes"] and d["record_state"] and not d["record_weights"] and not d["all_neurons"]


def test_result_reader(tmp_path):
    (tmp_path / "spikes.csv").write_text("time_step,component_kind,component_index,component_name,global_neuron_id,"
                                         "local_neuron_id\n3,main_network,0,main_network,7,7\n")
    (tmp_path / "meta.json").write_text('{"record_state": true}')
    r = open_debug_monitor(tmp_path)
    assert r.meta() == {"record_state": True}
    assert list(r.iter_rows("spikes")) == [{"time_step": "3", "component_kind": "main_network",
                                           "component_index": "0", "component_name": "main_network",
                                           "global_neuron_id": "7", "local_neuron_id": "7"}]
    assert r.file_sizes()["spikes"] > 0
    with pytest.raises(FileNotFoundError):
        r.table_path("weights")
    with pytest.raises(FileNotFoundError):
        DebugMonitorResult(tmp_path / "missing")
